// Multistep SCC / WCC on one GB300: trim, direction-optimising FW-BW
// reachability from a pivot, min-colour rounds to a fixed point; every label
// is its component's minimum vertex id when it is assigned.
//
// A run is one cooperative persistent kernel (k_run, all blocks resident)
// whose three phases are separated by grid barriers.  Each phase runs its
// whole level loop on the device: a "step" is a grid-strided pass over a
// frontier or candidate list ended by a bounded grid barrier, and the
// counters that steer the next step (frontier size, frontier edge count,
// deferred heavy vertices) rotate through three slots of the control block
// so that no block reads a counter another block is still writing.  The host
// never waits between levels.
//
// Reference phases (HPCGraphAnalysis/Connectivity, multistep/):
//   trim phase    scc_trim (scc_trim.cpp:89-139), scc_trim_complete
//                 (:141-297), cc_trim (cc_trim.cpp:47-97), pivot rule of
//                 create_csr (scc_main.cpp:169-182, cc_main.cpp:148-160)
//   reach phase   scc_fwbw_fw / scc_fwbw_bw / update_valid
//                 (scc_fwbw.cpp:47-466), cc_bfs_search / update_valid
//                 (cc_bfs.cpp:47-271)
//   colour phase  scc_color (scc_color.cpp:47-373) run until no vertex is
//                 left, which replaces the serial Tarjan step
//                 (scc_serial.cpp:160-258); cc_color_propagate
//                 (cc_color.cpp:47-175)
// This header holds the device code of a run; kernels.cu instantiates the
// default run kernels and kernels_options.cu the ones with the optional
// features compiled in.
#pragma once
#include "gb_internal.cuh"

namespace gb {
namespace {

// ------------------------------------------------------------------------
// Small device helpers
// ------------------------------------------------------------------------
__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }
__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned r;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
  return r;
}
__device__ __forceinline__ uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ int ld_vol(const int* p) { return *(volatile const int*)p; }

constexpr unsigned long long kBarErrBit = 1ull << 63;
__device__ __forceinline__ void set_err(Ctl* c, int code, int where) {
  if (atomicCAS(&c->err, 0, code) == 0) atomicExch(&c->err_where, where);
  // the barrier word carries the error too, so a barrier needs no second read
  atomicOr(&c->bar, kBarErrBit);
}

// Mutable arrays are read through L2 (ld.global.cg) so that a value written
// by another block in an earlier step is never served stale from L1.
__device__ __forceinline__ bool bit_get(const uint32_t* bm, int32_t v) {
  return (__ldcg(bm + (v >> 5)) >> (v & 31)) & 1u;
}
__device__ __forceinline__ bool bit_claim(uint32_t* bm, int32_t v) {
  const uint32_t b = 1u << (v & 31);
  return (atomicOr(bm + (v >> 5), b) & b) == 0u;
}
// L1-cacheable read for checks that tolerate a value from earlier in the
// same step (a stale "not set" only costs work: the atomic that follows, or
// the next step, settles it).  Values written before the last grid barrier
// are seen: the barrier's acquire by the block's first thread invalidates
// the SM's L1.
__device__ __forceinline__ bool bit_get_l1(const uint32_t* bm, int32_t v) {
  return (bm[v >> 5] >> (v & 31)) & 1u;
}
// Fire-and-forget set (RED): for bits only one thread can be setting.
__device__ __forceinline__ void bit_set_red(uint32_t* bm, int32_t v) {
  asm volatile("red.relaxed.gpu.global.or.b32 [%0], %1;" ::"l"(bm + (v >> 5)), "r"(1u << (v & 31))
               : "memory");
}
__device__ __forceinline__ bool bit_release(uint32_t* bm, int32_t v) {
  const uint32_t b = 1u << (v & 31);
  return (atomicAnd(bm + (v >> 5), ~b) & b) != 0u;
}

__device__ __forceinline__ long long shfl64(long long x, int src) {
  int lo = __shfl_sync(kFull, (int)(x & 0xffffffffll), src);
  int hi = __shfl_sync(kFull, (int)(x >> 32), src);
  return ((long long)hi << 32) | (unsigned)lo;
}
__device__ __forceinline__ unsigned long long warp_sum64(unsigned long long x) {
  for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(kFull, x, o);
  return x;
}
// Exclusive warp prefix sum; `total` receives the warp sum.
__device__ __forceinline__ int warp_excl(int x, int& total) {
  int inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(kFull, inc, o);
    if ((int)lane_id() >= o) inc += y;
  }
  total = __shfl_sync(kFull, inc, 31);
  return inc - x;
}

// Block-wide exclusive prefix sum over kBlock threads; returns the block
// total in `total`.  Contains __syncthreads.
__device__ int block_excl(int x, int& total, int* sm_warp /* kWarps + 1 */) {
  int wt;
  int ex = warp_excl(x, wt);
  const int warp = threadIdx.x >> 5;
  if (lane_id() == 31) sm_warp[warp] = wt;
  __syncthreads();
  if (warp == 0) {
    int v = (int)lane_id() < kWarps ? sm_warp[lane_id()] : 0;
    int t;
    int e = warp_excl(v, t);
    if ((int)lane_id() < kWarps) sm_warp[lane_id()] = e;
    if (lane_id() == 0) sm_warp[kWarps] = t;
  }
  __syncthreads();
  int r = ex + sm_warp[warp];
  total = sm_warp[kWarps];
  __syncthreads();
  return r;
}

constexpr unsigned long long kBarrierTimeoutNs = 20ull * 1000ull * 1000ull * 1000ull;
constexpr unsigned kBarrierMaxSpins = 1u << 28;

// Grid-wide barrier for a cooperative launch.  Thread 0 of every block adds
// one arrival to the barrier word and waits until the arrivals reach the
// next multiple of the grid size; the word's error bit ends every wait at
// once.  Every wait is bounded by time and by spin count; on expiry it sets
// the error.  Returns false when the kernel must stop.
__device__ __forceinline__ unsigned long long ld_acquire64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ bool grid_barrier(Ctl* c, int where) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned G = gridDim.x;
    const unsigned long long old = atomicAdd(&c->bar, 1ull);
    const unsigned arrived = (unsigned)old + 1u;
    const unsigned target = ((unsigned)old / G + 1u) * G;
    bool ok = (old & kBarErrBit) == 0ull;
    if (ok && arrived != target) {
      const uint64_t t0 = gtimer();
      unsigned spins = 0;
      for (;;) {
        const unsigned long long v = ld_acquire64(&c->bar);
        if (v & kBarErrBit) { ok = false; break; }
        if ((int)((unsigned)v - target) >= 0) break;
        __nanosleep(32);
        ++spins;
        if (spins >= kBarrierMaxSpins ||
            ((spins & 1023u) == 0u && gtimer() - t0 > kBarrierTimeoutNs)) {
          set_err(c, kErrTimeout, where);
          ok = false;
          break;
        }
      }
    }
    __threadfence();
    s_ok = ok ? 1 : 0;
  }
  __syncthreads();
  return s_ok != 0;
}

// Step bookkeeping: step s reads ring[s%3], appends into ring[(s+1)%3] and
// clears ring[(s+2)%3] (read two steps ago, written next step).  The step
// number persists in the control block across the kernels of one run, so
// the rotation continues over kernel boundaries.
struct StepIn {
  int32_t count, huge, cand;
  unsigned long long edges;
};
__device__ __forceinline__ StepIn step_read(Ctl* c, int step, int dir = 0) {
  const Slot& s = c->ring[step % 3][dir];
  StepIn r;
  r.count = __ldcg(&s.count);
  r.huge = __ldcg(&s.huge);
  r.cand = __ldcg(&s.cand);
  r.edges = __ldcg(&s.edges);
  return r;
}
__device__ __forceinline__ void step_begin(Ctl* c, int step) {
  if (blockIdx.x == 0 && threadIdx.x < 2) {
    Slot& s = c->ring[(step + 2) % 3][threadIdx.x];
    s.count = 0;
    s.huge = 0;
    s.cand = 0;
    s.edges = 0ull;
  }
}
__device__ __forceinline__ Slot* step_out(Ctl* c, int step, int dir = 0) {
  return &c->ring[(step + 1) % 3][dir];
}

constexpr unsigned long long kKernelTimeLimitNs = 120ull * 1000ull * 1000ull * 1000ull;

// Per-kernel step state: the step counter and the kernel's start time.  A
// kernel that runs past kKernelTimeLimitNs stops with kErrTimeout.
struct Steps {
  int s;
  int s0;
  uint64_t t0;
};
__device__ __forceinline__ Steps steps_open(Ctl* c) {
  Steps st;
  st.s = __ldcg(&c->step);
  st.s0 = st.s;
  st.t0 = gtimer();
  step_begin(c, st.s);
  return st;
}
// End the current step: barrier, next step number, clear the slot ahead.
__device__ __forceinline__ bool step_sync(Ctl* c, Steps& st, int where) {
  if (threadIdx.x == 0 && gtimer() - st.t0 > kKernelTimeLimitNs) set_err(c, kErrTimeout, 1000 + where);
  if (!grid_barrier(c, where)) return false;
  ++st.s;
  step_begin(c, st.s);
  return true;
}
__device__ __forceinline__ void steps_close(Ctl* c, const Steps& st) {
  if (st.s != st.s0 && blockIdx.x == 0 && threadIdx.x == 0) c->step = st.s;
}

// Per-thread counters of algorithmic traffic, flushed once per kernel.
struct Tally {
  unsigned long long vtx = 0, edges = 0, list = 0;
  unsigned long long pull_edges = 0;  // the part of `edges` scanned by pull steps
};
// Only statistics runs flush (the counters are summed per block first: one
// atomic per block and counter, not per warp, which would queue thousands of
// atomics on four words).  All threads of the block call it.
__device__ void tally_flush(const Tally& t, Ctl* c, int kernel, bool stats,
                            unsigned long long* red /* 4 x kWarps shared */) {
  if (!stats) return;
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const unsigned long long v[4] = {warp_sum64(t.vtx), warp_sum64(t.edges), warp_sum64(t.list),
                                   warp_sum64(t.pull_edges)};
  __syncthreads();
  if (lane_id() == 0)
    for (int k = 0; k < 4; ++k) red[k * kWarps + warp] = v[k];
  __syncthreads();
  if (threadIdx.x < 4) {
    unsigned long long x = 0ull;
    for (int i = 0; i < nw; ++i) x += red[threadIdx.x * kWarps + i];
    if (x) atomicAdd(threadIdx.x < 3 ? &c->kst[kernel][threadIdx.x] : &c->pull_edges, x);
  }
  __syncthreads();
}
// One trace record (block 0, thread 0).
__device__ __forceinline__ void trace_rec(Ctl* c, int32_t count, int32_t mode) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    auto& e = c->trace[c->ntrace % kTrace];
    e.t = gtimer();
    e.t_mid = 0;
    e.count = count;
    e.mode = mode;
    e.nwarp = 0;
    e.nblock = 0;
    c->ntrace++;
  }
}
__device__ __forceinline__ void stat_inc(Ctl* c, int slot) {
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&c->stat[slot], 1ull);
}

// Exclusive warp prefix sum in 64 bits.
__device__ __forceinline__ long long warp_excl64(long long x, long long& total) {
  long long inc = x;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long y = (long long)__shfl_up_sync(kFull, (unsigned long long)inc, o);
    if ((int)lane_id() >= o) inc += y;
  }
  total = (long long)__shfl_sync(kFull, (unsigned long long)inc, 31);
  return inc - x;
}
__device__ __forceinline__ int32_t warp_min(int32_t x) {
  for (int o = 16; o; o >>= 1) x = min(x, __shfl_xor_sync(kFull, x, o));
  return x;
}

// ------------------------------------------------------------------------
// Adjacency of a vertex over one or two CSRs (two: the union of out- and
// in-edges, which is the mirrored graph that cc builds, cc_main.cpp:102-118).
// The CSR arrays are read-only for a whole run (__ldg).
// ------------------------------------------------------------------------
// NC (1 or 2) is a compile-time copy of a.n, so the one-CSR paths carry no
// second-CSR state.
struct Adj {
  Csr c[2];
  int n;
};
template <int NC>
__device__ __forceinline__ void rec_load(const Adj& a, int32_t v, long long& s0, long long& d0,
                                         long long& s1, long long& d1) {
  s0 = __ldg(a.c[0].off + v);
  d0 = __ldg(a.c[0].off + v + 1) - s0;
  s1 = 0;
  d1 = 0;
  if constexpr (NC > 1) {
    s1 = __ldg(a.c[1].off + v);
    d1 = __ldg(a.c[1].off + v + 1) - s1;
  }
}
template <int NC>
__device__ __forceinline__ int32_t adj_at(const Adj& a, long long s0, long long d0, long long s1,
                                          long long e, int& k) {
  if constexpr (NC == 1) {
    k = 0;
    return __ldg(a.c[0].adj + s0 + e);
  } else {
    if (e < d0) {
      k = 0;
      return __ldg(a.c[0].adj + s0 + e);
    }
    k = 1;
    return __ldg(a.c[1].adj + s1 + (e - d0));
  }
}
template <int NC>
__device__ __forceinline__ unsigned long long adj_degree(const Adj& a, int32_t v) {
  long long d = __ldg(a.c[0].off + v + 1) - __ldg(a.c[0].off + v);
  if constexpr (NC > 1) d += __ldg(a.c[1].off + v + 1) - __ldg(a.c[1].off + v);
  return (unsigned long long)d;
}
__device__ __forceinline__ Adj adj1(Csr x) {
  Adj a;
  a.c[0] = x;
  a.c[1] = x;
  a.n = 1;
  return a;
}
__device__ __forceinline__ Adj adj2(Csr x, Csr y) {
  Adj a;
  a.c[0] = x;
  a.c[1] = y;
  a.n = 2;
  return a;
}
// Undirected view: the union of both CSRs of a directed graph, or the single
// CSR of a symmetric one.
__device__ __forceinline__ Adj adj_undirected(const GraphView& g) {
  return g.in.off != nullptr ? adj2(g.out, g.in) : adj1(g.out);
}

// ------------------------------------------------------------------------
// Appends.  Each warp stages the vertices it appends in shared memory and
// moves them to the global list in one atomic + coalesced copy per kWB
// entries, which keeps the step counters (a single L2 word) cool.
// ------------------------------------------------------------------------
constexpr int kWB = 256;
// Per-warp backlog of pull candidates the hint did not settle (entries).
constexpr int kTodo = 384;
// Dynamic shared memory of the cooperative kernels: two staging buffers and
// one pull backlog per warp.
constexpr int kWarpSmem = 2 * kWB + kTodo;
constexpr int kDynSmem = kWarps * kWarpSmem * 4;
// a warp's shared memory also holds the ids of 16 bitmap words
static_assert(kWB * 2 + kTodo >= 16 * 32, "warp shared memory too small for 16 words");

// A global output list.
struct Out {
  int32_t* arr;               // receives vertices at base + slot
  long long base;
  long long cap;              // bound on base + slot
  int32_t* counter;           // slot counter
  unsigned long long* edges;  // weight sum, or null
  int32_t* minv;              // smallest appended id, or null
  int where;                  // error site
};

// One warp's staging buffer for one Out (n is warp-uniform).
struct Stage {
  int32_t* buf;
  int n;
  unsigned long long wsum;
  int32_t vmin;
};
__device__ __forceinline__ Stage stage_make(int32_t* buf) {
  Stage s;
  s.buf = buf;
  s.n = 0;
  s.wsum = 0ull;
  s.vmin = 0x7fffffff;
  return s;
}
// All 32 lanes call.
__device__ __noinline__ void stage_flush(Stage& s, const Out& o, Ctl* c) {
  __syncwarp();
  const int lane = lane_id();
  if (s.n > 0) {
    int pos = 0;
    if (lane == 0) pos = atomicAdd(o.counter, s.n);
    pos = __shfl_sync(kFull, pos, 0);
    for (int i = lane; i < s.n; i += 32) {
      const long long at = o.base + pos + i;
      if (at < o.cap) o.arr[at] = s.buf[i];
      else set_err(c, kErrCapacity, o.where);
    }
  }
  if (o.edges != nullptr) {
    const unsigned long long ws = warp_sum64(s.wsum);
    if (lane == 0 && ws) atomicAdd(o.edges, ws);
  }
  if (o.minv != nullptr) {
    const int32_t mn = warp_min(s.vmin);
    if (lane == 0 && mn != 0x7fffffff) atomicMin(o.minv, mn);
  }
  __syncwarp();
  s.n = 0;
  s.wsum = 0ull;
  s.vmin = 0x7fffffff;
}
// All 32 lanes call; lanes with `flag` append v (weight wt).
__device__ __forceinline__ void stage_push(Stage& s, bool flag, int32_t v, unsigned long long wt,
                                           const Out& o, Ctl* c) {
  const unsigned mask = __ballot_sync(kFull, flag);
  if (mask == 0u) return;
  const int cnt = __popc(mask);
  if (s.n + cnt > kWB) stage_flush(s, o, c);
  if (flag) {
    s.buf[s.n + __popc(mask & lanemask_lt())] = v;
    s.wsum += wt;
    s.vmin = min(s.vmin, v);
  }
  s.n += cnt;
}

// Plain warp-aggregated append (used for the rare heavy-vertex lists).
__device__ __forceinline__ void list_append(bool app, int32_t v, int32_t* arr, int32_t* counter,
                                            long long cap, Ctl* c, int where) {
  const unsigned mask = __ballot_sync(kFull, app);
  if (mask == 0u) return;
  const int leader = __ffs(mask) - 1;
  int pos = 0;
  if ((int)lane_id() == leader) pos = atomicAdd(counter, __popc(mask));
  pos = __shfl_sync(kFull, pos, leader) + __popc(mask & lanemask_lt());
  if (app) {
    if (pos < cap) arr[pos] = v;
    else set_err(c, kErrCapacity, where);
  }
}

struct BlockList {
  int cnt;
  int32_t v[kBlkList];
  int32_t sval[kBlkList];
  long long s0[kBlkList];
  long long d0[kBlkList];
  long long s1[kBlkList];
  long long d1[kBlkList];
};

struct Smem {
  BlockList bl;
  int warp_tmp[kWarps + 1];
  long long red_l[kWarps];
  unsigned long long red_u[4 * kWarps];  // statistics tallies, per warp
  int red_i[kWarps];
  // dynamic shared memory: per warp, contiguous, two staging buffers of kWB
  // entries then a pull backlog of kTodo entries (kWarpSmem entries in all)
  int32_t* stage_base;
  __device__ __forceinline__ int32_t* stage(int warp, int k) {
    return stage_base + warp * kWarpSmem + k * kWB;
  }
  __device__ __forceinline__ int32_t* todo(int warp) {
    return stage_base + warp * kWarpSmem + 2 * kWB;
  }
};
extern __shared__ __align__(16) int32_t g_dyn_smem[];

// Output of one expansion step: the main list and the heavy list.
struct Sink {
  Out out;
  int32_t* harr;              // heavy list for the next step, or null
  int32_t hcap;
  int32_t* hcounter;
};
__device__ __forceinline__ Sink sink_make(int32_t* arr, long long base, long long cap, Slot* o,
                                          bool weighted, int32_t* minv, int32_t* harr,
                                          int32_t hcap, int where) {
  Sink k;
  k.out.arr = arr;
  k.out.base = base;
  k.out.cap = cap;
  k.out.counter = &o->count;
  k.out.edges = weighted ? &o->edges : nullptr;
  k.out.minv = minv;
  k.out.where = where;
  k.harr = harr;
  k.hcap = hcap;
  k.hcounter = &o->huge;
  return k;
}

// Visits kEU edges per lane at once: the visitor issues the loads of all of
// them, then their atomics, so the memory latencies overlap; the far ends it
// accepts are appended.
constexpr int kEU = 4;
template <class V>
__device__ __forceinline__ void visit_edges(const V& vis, const int32_t (&sv)[kEU],
                                            const int32_t (&w)[kEU], const int (&k)[kEU],
                                            const bool (&act)[kEU], Stage& st, const Sink& sk,
                                            Ctl* c) {
  bool app[kEU];
  vis.edges(sv, w, k, act, app);
  unsigned long long wt[kEU];
#pragma unroll
  for (int q = 0; q < kEU; ++q)
    wt[q] = (V::kWeighted && app[q] && sk.out.edges != nullptr) ? vis.weight(w[q]) : 0ull;
#pragma unroll
  for (int q = 0; q < kEU; ++q) stage_push(st, app[q], w[q], wt[q], sk.out, c);
}

constexpr int kSmallFront = 8;
constexpr int kLocalRounds = 32;       // local rounds per step
constexpr long long kLocalDegree = 4096;  // heavier vertices go to the next step

// Local rounds (visitors with kLocal): the vertices this warp appended in
// its stage are expanded by the warp itself, up to kLocalRounds rounds, so a
// propagation runs several hops per grid step.  Every acceptance hands its
// vertex to exactly one warp (the colour visitor: each successful lowering;
// the mark visitor: each claim), and that warp either expands it here, with
// the vertex's value read now, or appends it for the next step, so nothing
// is lost.  A vertex heavier than kLocalDegree goes to the next step.
template <int NC, class V>
__device__ __forceinline__ void local_rounds(const Adj& a, const V& vis, Stage& st,
                                             const Sink& sk, Smem& sm, Ctl* c, Tally& ty) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int32_t* loc = sm.stage(warp, 1);  // free in push steps: kWB entries
  for (int r = 0; r < kLocalRounds; ++r) {
    const int cnt = st.n;  // warp-uniform, at most kWB
    if (cnt == 0) break;
    __syncwarp();
    for (int i = lane; i < cnt; i += 32) loc[i] = st.buf[i];
    __syncwarp();
    st.n = 0;
    for (int b0 = 0; b0 < cnt; b0 += 32) {
      const int i = b0 + lane;
      const int32_t v = i < cnt ? loc[i] : -1;
      long long s0 = 0, d0 = 0, s1 = 0, d1 = 0;
      if (v >= 0) {
        rec_load<NC>(a, v, s0, d0, s1, d1);
        ty.vtx += NC;
        ty.list++;
      }
      const long long d = d0 + d1;
      const bool heavy = v >= 0 && d > kLocalDegree;
      list_append(heavy, v, sk.out.arr + sk.out.base, sk.out.counter, sk.out.cap - sk.out.base, c,
                  304);
      const long long mine = (v >= 0 && !heavy) ? d : 0;
      const int32_t sv = mine ? vis.source(v) : 0;
      long long tot;
      const long long ex = warp_excl64(mine, tot);
      for (long long eb = 0; eb < tot; eb += 32 * kEU) {
        int32_t svq[kEU], w[kEU];
        int k[kEU];
        bool act[kEU];
#pragma unroll
        for (int q = 0; q < kEU; ++q) {
          const long long e = eb + q * 32 + lane;
          act[q] = e < tot;
          int j = 0;
#pragma unroll
          for (int stp = 16; stp; stp >>= 1) {
            const int cnd = j + stp;
            const long long exc = shfl64(ex, cnd);
            if (exc <= e) j = cnd;
          }
          const long long ej = shfl64(ex, j);
          svq[q] = __shfl_sync(kFull, sv, j);
          const long long s0j = shfl64(s0, j), d0j = shfl64(d0, j), s1j = shfl64(s1, j);
          w[q] = 0;
          k[q] = 0;
          if (act[q]) {
            w[q] = adj_at<NC>(a, s0j, d0j, s1j, e - ej, k[q]);
            ty.edges++;
          }
        }
        visit_edges(vis, svq, w, k, act, st, sk, c);
      }
    }
  }
}

// ------------------------------------------------------------------------
// Frontier expansion (push).  Three tiers by degree:
//   d >= t_grid : deferred to the next step, where every block takes a
//                 1/grid slice of the vertex's edges;
//   d >= t_block: the whole block walks the edges (per-block list);
//   otherwise   : a warp takes 32 vertices (fewer when the frontier is
//                 smaller than 32 per warp of the grid: then every warp
//                 gets a share, and with it its own chain of local rounds),
//                 scans their degrees and walks the concatenated edge lists
//                 32 edges at a time.
// A frontier of at most kSmallFront vertices is sliced across all blocks in
// the same step.  The visitor decides per edge whether the far end is
// appended.  Ends with every warp's staging flushed.
// ------------------------------------------------------------------------
template <int NC, class V>
__device__ void expand(const int32_t* front, int32_t nfront, const int32_t* heavy, int32_t nheavy,
                       const Adj& a, const V& vis, const Sink& sk, const Tune& tn, Smem& sm,
                       Ctl* c, Tally& ty) {
  const int G = gridDim.x, b = blockIdx.x, T = blockDim.x, t = threadIdx.x;
  const int warp = t >> 5, lane = t & 31;
  Stage st = stage_make(sm.stage(warp, 0));
  const bool small = nfront <= kSmallFront;
  // (1) heavy vertices deferred by the previous step, and a small frontier.
  // Their records are loaded in parallel, 32 at a time, into shared memory;
  // a vertex of degree >= t_block is cut into one slice per block, a lighter
  // one is walked by the single block (index mod grid size) that owns it.
  const int nsl = nheavy + (small ? nfront : 0);
  for (int j0 = 0; j0 < nsl; j0 += 32) {
    __syncthreads();
    if (warp == 0) {
      const int j = j0 + lane;
      if (j < nsl) {
        const int32_t v = j < nheavy ? __ldcg(heavy + j) : __ldcg(front + (j - nheavy));
        long long s0, d0, s1, d1;
        rec_load<NC>(a, v, s0, d0, s1, d1);
        sm.bl.v[lane] = v;
        sm.bl.sval[lane] = vis.source(v);
        sm.bl.s0[lane] = s0;
        sm.bl.d0[lane] = d0;
        sm.bl.s1[lane] = s1;
        sm.bl.d1[lane] = d1;
      }
    }
    __syncthreads();
    const int cnt = nsl - j0 < 32 ? nsl - j0 : 32;
    for (int jj = 0; jj < cnt; ++jj) {
      const long long s0 = sm.bl.s0[jj], d0 = sm.bl.d0[jj], s1 = sm.bl.s1[jj];
      const long long d = d0 + sm.bl.d1[jj];
      const int32_t sv = sm.bl.sval[jj];
      long long lo = 0, hi = d;
      if (d >= tn.t_block) {
        lo = d * b / G;
        hi = d * (b + 1) / G;
      } else if ((j0 + jj) % G != b) {
        continue;
      }
      if (t == 0 && (b == 0 || d < tn.t_block)) ty.vtx += NC;
      for (long long e0 = lo; e0 < hi; e0 += (long long)T * kEU) {
        int32_t svq[kEU], w[kEU];
        int k[kEU];
        bool act[kEU];
#pragma unroll
        for (int q = 0; q < kEU; ++q) {
          const long long e = e0 + (long long)q * T + t;
          act[q] = e < hi;
          svq[q] = sv;
          w[q] = 0;
          k[q] = 0;
          if (act[q]) {
            w[q] = adj_at<NC>(a, s0, d0, s1, e, k[q]);
            ty.edges++;
          }
        }
        visit_edges(vis, svq, w, k, act, st, sk, c);
      }
    }
  }
  if (small) {
    if constexpr (V::kLocal) {
      if (vis.local()) local_rounds<NC>(a, vis, st, sk, sm, c, ty);
    }
    stage_flush(st, sk.out, c);
    return;
  }
  // (2) regular frontier, warp-gathered
  if (t == 0) sm.bl.cnt = 0;
  __syncthreads();
  const long long nw = (long long)G * (T >> 5);
  // a frontier smaller than 32 per warp is spread over all warps
  const int vpw = (long long)nfront >= nw * 32 ? 32 : (int)(((long long)nfront + nw - 1) / nw);
  for (long long base = ((long long)b * (T >> 5) + warp) * vpw; base < nfront; base += nw * vpw) {
    const long long i = base + lane;
    int32_t v = -1;
    long long s0 = 0, d0 = 0, s1 = 0, d1 = 0;
    if (lane < vpw && i < nfront) {
      v = __ldcg(front + i);
      rec_load<NC>(a, v, s0, d0, s1, d1);
      ty.list++;
      ty.vtx += NC;
    }
    const long long d = d0 + d1;
    const bool to_grid = v >= 0 && d >= tn.t_grid && sk.harr != nullptr;
    list_append(to_grid, v, sk.harr, sk.hcounter, sk.hcap, c, 102);
    bool to_block = false;
    if (v >= 0 && !to_grid && d >= tn.t_block) {
      const int slot = atomicAdd(&sm.bl.cnt, 1);
      if (slot < kBlkList) {
        sm.bl.v[slot] = v;
        sm.bl.sval[slot] = vis.source(v);
        sm.bl.s0[slot] = s0;
        sm.bl.d0[slot] = d0;
        sm.bl.s1[slot] = s1;
        sm.bl.d1[slot] = d1;
        to_block = true;
      }
    }
    const long long mine = (v < 0 || to_grid || to_block) ? 0 : d;
    const int32_t sv = mine ? vis.source(v) : 0;
    long long tot;
    const long long ex = warp_excl64(mine, tot);
    for (long long eb = 0; eb < tot; eb += 32 * kEU) {
      int32_t svq[kEU], w[kEU];
      int k[kEU];
      bool act[kEU];
#pragma unroll
      for (int q = 0; q < kEU; ++q) {
        const long long e = eb + q * 32 + lane;
        act[q] = e < tot;
        // the owner of edge e: the last lane whose exclusive prefix is <= e
        int j = 0;
#pragma unroll
        for (int stp = 16; stp; stp >>= 1) {
          const int cnd = j + stp;
          const long long exc = shfl64(ex, cnd);
          if (exc <= e) j = cnd;
        }
        const long long ej = shfl64(ex, j);
        svq[q] = __shfl_sync(kFull, sv, j);
        const long long s0j = shfl64(s0, j), d0j = shfl64(d0, j), s1j = shfl64(s1, j);
        w[q] = 0;
        k[q] = 0;
        if (act[q]) {
          w[q] = adj_at<NC>(a, s0j, d0j, s1j, e - ej, k[q]);
          ty.edges++;
        }
      }
      visit_edges(vis, svq, w, k, act, st, sk, c);
    }
  }
  __syncthreads();
  // (3) block-expanded vertices
  const int nb = sm.bl.cnt < kBlkList ? sm.bl.cnt : kBlkList;
  for (int j = 0; j < nb; ++j) {
    const int32_t sv = sm.bl.sval[j];
    const long long s0 = sm.bl.s0[j], d0 = sm.bl.d0[j], s1 = sm.bl.s1[j];
    const long long d = d0 + sm.bl.d1[j];
    for (long long e0 = 0; e0 < d; e0 += (long long)T * kEU) {
      int32_t svq[kEU], w[kEU];
      int k[kEU];
      bool act[kEU];
#pragma unroll
      for (int q = 0; q < kEU; ++q) {
        const long long e = e0 + (long long)q * T + t;
        act[q] = e < d;
        svq[q] = sv;
        w[q] = 0;
        k[q] = 0;
        if (act[q]) {
          w[q] = adj_at<NC>(a, s0, d0, s1, e, k[q]);
          ty.edges++;
        }
      }
      visit_edges(vis, svq, w, k, act, st, sk, c);
    }
  }
  if constexpr (V::kLocal) {
    if (vis.local()) local_rounds<NC>(a, vis, st, sk, sm, c, ty);
  }
  stage_flush(st, sk.out, c);
  __syncthreads();
}

// ------------------------------------------------------------------------
// Global edge-balanced push (Tune::expand_mode 1): the Kokkos variant's
// "manhattan global" scheme (kokkos_scc/fwbw_manhattan_global.cpp:186-289),
// restated for this kernel as an alternative to the degree tiers.  The
// frontier's edges are numbered in frontier order and every warp of the grid
// takes an equal contiguous share of the numbers, so no vertex is deferred
// and no tier decides who walks it.  The numbering needs the frontier's
// degree prefix: each block sums the 32-vertex groups of its contiguous
// share of the frontier (group prefixes local to the block go to `pre`, the
// block's total to btot[b]); one grid barrier publishes the totals; each
// warp then finds the group of its first edge (a scan of the block totals,
// then a binary search over that block's group prefixes) and walks group by
// group to the end of its share.  Every warp of the grid reads the block
// totals, and with a small frontier the same few groups: those reads go
// through L1 (values written before the last grid barrier are seen, since
// the barrier's acquire invalidates the SM's L1), so that one L2 request per
// SM, not one per warp, serves them.  Returns false when the kernel must
// stop.
// ------------------------------------------------------------------------
template <int NC, class V>
__device__ __noinline__ bool expand_balanced(const int32_t* front, int32_t nfront, const Adj& a,
                                             const V& vis, const Sink& sk,
                                             long long* pre /* >= ceil(nfront / 32) */,
                                             long long* btot /* grid size */, Smem& sm, Ctl* c,
                                             Tally& ty) {
  const int G = gridDim.x, b = blockIdx.x, T = blockDim.x, t = threadIdx.x;
  const int warp = t >> 5, lane = t & 31, nwarps = T >> 5;
  Stage st = stage_make(sm.stage(warp, 0));
  const long long ngroups = ((long long)nfront + 31) / 32;
  const long long gpb = (ngroups + G - 1) / G;
  const long long g0 = gpb * b < ngroups ? gpb * b : ngroups;
  const long long g1 = g0 + gpb < ngroups ? g0 + gpb : ngroups;
  // (a) the block's groups, one per warp per round: sums, then a block scan
  long long run = 0;  // the block's edges before this round (same in every thread)
  for (long long r0 = g0; r0 < g1; r0 += nwarps) {
    const long long gi = r0 + warp;
    long long d = 0;
    if (gi < g1 && gi * 32 + lane < nfront) {
      d = (long long)adj_degree<NC>(a, __ldcg(front + gi * 32 + lane));
      ty.vtx += NC;
    }
    const long long gsum = warp_sum64(d);
    __syncthreads();
    if (lane == 0) sm.red_l[warp] = gsum;
    __syncthreads();
    if (warp == 0) {
      const long long x = lane < nwarps ? sm.red_l[lane] : 0;
      long long tot;
      const long long ex = warp_excl64(x, tot);
      if (lane < nwarps) sm.red_l[lane] = ex;
      if (lane == 0) sm.red_u[0] = (unsigned long long)tot;
    }
    __syncthreads();
    if (gi < g1 && lane == 0) pre[gi] = run + sm.red_l[warp];
    run += (long long)sm.red_u[0];
  }
  if (t == 0) btot[b] = run;
  if (!grid_barrier(c, 210)) return false;
  // (b) the block totals' prefix, per warp: lane L holds blocks
  // [L * per, (L + 1) * per)
  const int per = (G + 31) / 32;
  long long lsum = 0;
  for (int j = 0; j < per; ++j) {
    const int bb = lane * per + j;
    if (bb < G) lsum += btot[bb];
  }
  long long E;
  const long long lpre = warp_excl64(lsum, E);
  const long long W = (long long)G * nwarps;
  const long long gw = (long long)b * nwarps + warp;
  const long long e0 = E * gw / W, e1 = E * (gw + 1) / W;
  if (e0 < e1) {
    // the block whose edges hold e0
    int blk = -1;
    long long bstart = 0;
    {
      long long p = lpre;
      for (int j = 0; j < per; ++j) {
        const int bb = lane * per + j;
        const long long tb = bb < G ? btot[bb] : 0;
        if (tb > 0 && p <= e0 && e0 < p + tb) {
          blk = bb;
          bstart = p;
        }
        p += tb;
      }
    }
    const unsigned m = __ballot_sync(kFull, blk >= 0);
    const int src = __ffs(m) - 1;  // exactly one lane holds it (e0 < E)
    blk = __shfl_sync(kFull, blk, src);
    bstart = shfl64(bstart, src);
    // the last group of that block whose local prefix is <= e0 - bstart
    const long long x = e0 - bstart;
    long long lo = gpb * blk, hi = gpb * blk + gpb < ngroups ? gpb * blk + gpb : ngroups;
    while (hi - lo > 1) {
      const long long mid = (lo + hi) >> 1;
      if (pre[mid] <= x) lo = mid;
      else hi = mid;
    }
    long long gi = lo;
    long long P = bstart + pre[gi];  // global number of the group's first edge
    // (c) walk the groups from there to the end of this warp's share
    while (P < e1 && gi < ngroups) {
      const long long i = gi * 32 + lane;
      long long s0 = 0, d0 = 0, s1 = 0, d1 = 0;
      int32_t v = -1;
      if (i < nfront) {
        v = front[i];
        rec_load<NC>(a, v, s0, d0, s1, d1);
        ty.list++;
      }
      const int32_t sv = v >= 0 ? vis.source(v) : 0;
      long long tot;
      const long long ex = warp_excl64(d0 + d1, tot);
      const long long lo_e = (e0 > P ? e0 : P) - P;
      const long long hi_e = (e1 < P + tot ? e1 : P + tot) - P;
      for (long long eb = lo_e; eb < hi_e; eb += 32 * kEU) {
        int32_t svq[kEU], w[kEU];
        int k[kEU];
        bool act[kEU];
#pragma unroll
        for (int q = 0; q < kEU; ++q) {
          const long long e = eb + q * 32 + lane;
          act[q] = e < hi_e;
          // the owner of edge e: the last lane whose exclusive prefix is <= e
          int j = 0;
#pragma unroll
          for (int stp = 16; stp; stp >>= 1) {
            const int cnd = j + stp;
            const long long exc = shfl64(ex, cnd);
            if (exc <= e) j = cnd;
          }
          const long long ej = shfl64(ex, j);
          svq[q] = __shfl_sync(kFull, sv, j);
          const long long s0j = shfl64(s0, j), d0j = shfl64(d0, j), s1j = shfl64(s1, j);
          w[q] = 0;
          k[q] = 0;
          if (act[q]) {
            w[q] = adj_at<NC>(a, s0j, d0j, s1j, e - ej, k[q]);
            ty.edges++;
          }
        }
        visit_edges(vis, svq, w, k, act, st, sk, c);
      }
      P += tot;
      ++gi;
    }
  }
  if constexpr (V::kLocal) {
    if (vis.local()) local_rounds<NC>(a, vis, st, sk, sm, c, ty);
  }
  stage_flush(st, sk.out, c);
  __syncthreads();
  return true;
}

// ------------------------------------------------------------------------
// Visitors: edge(source value, far end, which CSR, active) -> append?
// ------------------------------------------------------------------------
// Reachability: the far end is taken if allowed and not yet reached.
template <int NC>
struct ReachVisit {
  static constexpr bool kWeighted = true;
  static constexpr bool kLocal = true;
  const uint32_t* allow;
  uint32_t* vis;
  Adj push;
  bool local_ok;  // this search may expand its claims in local rounds
  __device__ __forceinline__ bool local() const { return local_ok; }
  __device__ __forceinline__ int32_t source(int32_t) const { return 0; }
  __device__ __forceinline__ void edges(const int32_t (&)[kEU], const int32_t (&w)[kEU],
                                        const int (&)[kEU], const bool (&act)[kEU],
                                        bool (&out)[kEU]) const {
    bool p[kEU];
#pragma unroll
    for (int q = 0; q < kEU; ++q) {
      const bool seen = bit_get_l1(vis, w[q]);
      const bool ok = bit_get_l1(allow, w[q]);
      p[q] = act[q] && !seen && ok;
    }
#pragma unroll
    for (int q = 0; q < kEU; ++q) out[q] = p[q] && bit_claim(vis, w[q]);
  }
  __device__ __forceinline__ unsigned long long weight(int32_t w) const {
    return adj_degree<NC>(push, w);
  }
};

// Colour push: colour[w] = min(colour[w], colour[v]) over valid w.  The
// reference pushes the maximum (scc_color.cpp:89-113, cc_color.cpp:103-127);
// pushing the minimum is the same algorithm mirrored, and its roots are the
// smallest ids of their SCCs, so the labels come out canonical.  Every
// lowering that succeeds hands w on (to the lowering warp's local rounds or
// to the next step), so a vertex lowered twice in a step is pushed twice,
// each time with its colour at that moment.
struct ColourVisit {
  static constexpr bool kWeighted = false;
  static constexpr bool kLocal = true;
  const uint32_t* valid;
  int32_t* colour;
  __device__ __forceinline__ bool local() const { return true; }
  __device__ __forceinline__ int32_t source(int32_t v) const { return __ldcg(colour + v); }
  __device__ __forceinline__ void edges(const int32_t (&cv)[kEU], const int32_t (&w)[kEU],
                                        const int (&)[kEU], const bool (&act)[kEU],
                                        bool (&out)[kEU]) const {
    bool p[kEU];
#pragma unroll
    for (int q = 0; q < kEU; ++q) {
      const bool ok = bit_get(valid, w[q]);
      const int32_t cw = __ldcg(colour + w[q]);
      p[q] = act[q] && ok && cw > cv[q];
    }
    int32_t m[kEU];
#pragma unroll
    for (int q = 0; q < kEU; ++q) m[q] = p[q] ? atomicMin(colour + w[q], cv[q]) : cv[q];
#pragma unroll
    for (int q = 0; q < kEU; ++q) out[q] = p[q] && m[q] > cv[q];
  }
  __device__ __forceinline__ unsigned long long weight(int32_t) const { return 0ull; }
};

// Backward search inside one colour (scc_color_find_sccs,
// scc_color.cpp:243-252): a valid in-neighbour with the same colour joins the
// root's SCC and is labelled with the colour.
struct MarkVisit {
  static constexpr bool kWeighted = false;
  static constexpr bool kLocal = true;
  __device__ __forceinline__ bool local() const { return true; }
  const uint32_t* valid;
  uint32_t* done;
  const int32_t* colour;
  int32_t* label;
  __device__ __forceinline__ int32_t source(int32_t v) const { return __ldcg(colour + v); }
  __device__ __forceinline__ void edges(const int32_t (&cv)[kEU], const int32_t (&u)[kEU],
                                        const int (&)[kEU], const bool (&act)[kEU],
                                        bool (&out)[kEU]) const {
    bool p[kEU];
#pragma unroll
    for (int q = 0; q < kEU; ++q) {
      const bool ok = bit_get(valid, u[q]);
      const int32_t cu = __ldcg(colour + u[q]);
      const bool dn = bit_get(done, u[q]);
      p[q] = act[q] && ok && cu == cv[q] && !dn;
    }
#pragma unroll
    for (int q = 0; q < kEU; ++q) out[q] = p[q] && bit_claim(done, u[q]);
#pragma unroll
    for (int q = 0; q < kEU; ++q)
      if (out[q]) label[u[q]] = cv[q];
  }
  __device__ __forceinline__ unsigned long long weight(int32_t) const { return 0ull; }
};

// Signature propagation (colour_mode 1): the visited vertex's value (the
// smallest id reaching it, or reached from it) is lowered along an edge that
// stays inside its class (both ends carried the same value pair in the
// previous round).  The source value is the vertex itself: its value and
// class are read here.
struct SigVisit {
  static constexpr bool kWeighted = false;
  static constexpr bool kLocal = true;
  const uint32_t* valid;
  int32_t* val;
  const int32_t* cls;
  __device__ __forceinline__ bool local() const { return true; }
  __device__ __forceinline__ int32_t source(int32_t v) const { return v; }
  __device__ __forceinline__ void edges(const int32_t (&sv)[kEU], const int32_t (&w)[kEU],
                                        const int (&)[kEU], const bool (&act)[kEU],
                                        bool (&out)[kEU]) const {
    bool p[kEU];
    int32_t cv[kEU];
#pragma unroll
    for (int q = 0; q < kEU; ++q) {
      p[q] = act[q] && bit_get(valid, w[q]);
      cv[q] = 0;
      if (p[q]) {
        cv[q] = __ldcg(val + sv[q]);
        p[q] = __ldcg(cls + sv[q]) == __ldcg(cls + w[q]) && __ldcg(val + w[q]) > cv[q];
      }
    }
    int32_t m[kEU];
#pragma unroll
    for (int q = 0; q < kEU; ++q) m[q] = p[q] ? atomicMin(val + w[q], cv[q]) : cv[q];
#pragma unroll
    for (int q = 0; q < kEU; ++q) out[q] = p[q] && m[q] > cv[q];
  }
  __device__ __forceinline__ unsigned long long weight(int32_t) const { return 0ull; }
};

// Fixed-point trim: removing r takes one edge from each neighbour's live
// count (out-edge r->w: w loses an in-edge; in-edge u->r: u loses an
// out-edge).  A valid vertex whose count reaches zero is removed and labelled
// with itself (scc_trim_complete, scc_trim.cpp:205-263).
struct TrimVisit {
  static constexpr bool kWeighted = false;
  static constexpr bool kLocal = false;
  uint32_t* valid;
  int32_t* live_in;
  int32_t* live_out;
  int32_t* label;
  __device__ __forceinline__ int32_t source(int32_t) const { return 0; }
  __device__ __forceinline__ void edges(const int32_t (&)[kEU], const int32_t (&w)[kEU],
                                        const int (&k)[kEU], const bool (&act)[kEU],
                                        bool (&out)[kEU]) const {
    bool p[kEU];
#pragma unroll
    for (int q = 0; q < kEU; ++q) p[q] = act[q] && bit_get(valid, w[q]);
    int32_t r[kEU];
#pragma unroll
    for (int q = 0; q < kEU; ++q) r[q] = p[q] ? atomicSub((k[q] == 0 ? live_in : live_out) + w[q], 1) : 0;
#pragma unroll
    for (int q = 0; q < kEU; ++q) out[q] = p[q] && r[q] == 1 && bit_release(valid, w[q]);
#pragma unroll
    for (int q = 0; q < kEU; ++q)
      if (out[q]) label[w[q]] = w[q];
  }
  __device__ __forceinline__ unsigned long long weight(int32_t) const { return 0ull; }
};

// ------------------------------------------------------------------------
// Kernel arguments
// ------------------------------------------------------------------------
struct Args {
  GraphView g;
  RunParams p;
  Work w;
  int kind;
};

// Ordered compaction: in[0, nin) -> out, keeping the entries whose bit is
// clear in `drop`, in list order.  Block b owns a contiguous chunk; one
// barrier between counting and writing.  The survivor count goes to *total.
template <class F>
__device__ bool compact_ordered(const int32_t* in, int32_t nin, int32_t* out, const uint32_t* drop,
                                Work& w, Smem& sm, Steps& st, int where, int32_t* total,
                                Tally& ty, F on_drop) {
  // Every warp owns a contiguous range (ranges follow the global warp
  // order): pass 1 counts what stays and hands every dropped element to
  // on_drop, one grid barrier publishes the block totals, pass 2 writes
  // with warp ballots.  kCU elements per lane per iteration keep the loads
  // overlapped.
  constexpr int kCU = 8;
  constexpr long long kCG = 32 * kCU;
  const int G = gridDim.x, b = blockIdx.x, T = blockDim.x, t = threadIdx.x;
  const int warp = t >> 5, lane = t & 31, nwarps = T >> 5;
  const long long W = (long long)G * nwarps;
  const long long gw = (long long)b * nwarps + warp;
  const long long wchunk = (((long long)nin + W - 1) / W + 31) / 32 * 32;
  const long long wlo = wchunk * gw < nin ? wchunk * gw : nin;
  const long long whi = wlo + wchunk < nin ? wlo + wchunk : nin;
  int cnt = 0;  // warp-uniform
  for (long long base = wlo; base < whi; base += kCG) {
    int32_t v[kCU];
#pragma unroll
    for (int j = 0; j < kCU; ++j) {
      const long long i = base + j * 32 + lane;
      v[j] = i < whi ? __ldcg(in + i) : -1;
    }
#pragma unroll
    for (int j = 0; j < kCU; ++j) {
      const bool d = v[j] >= 0 && bit_get(drop, v[j]);
      if (d) on_drop(v[j]);
      if (v[j] >= 0) ty.list++;
      cnt += __popc(__ballot_sync(kFull, v[j] >= 0 && !d));
    }
  }
  // warp offsets inside the block, block total
  __syncthreads();
  if (lane == 0) sm.warp_tmp[warp] = cnt;
  __syncthreads();
  if (warp == 0) {
    const int x = lane < nwarps ? sm.warp_tmp[lane] : 0;
    int incl = x;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const int y = __shfl_up_sync(kFull, incl, d);
      if (lane >= d) incl += y;
    }
    if (lane < nwarps) sm.warp_tmp[lane] = incl - x;
    if (lane == 31) w.blk_i[b] = incl;
  }
  __syncthreads();
  const int woff = sm.warp_tmp[warp];
  if (!step_sync(w.ctl, st, where)) return false;
  int pre = 0;
  for (int j = t; j < b; j += T) pre += __ldcg(w.blk_i + j);
  const int tot = __ldcg(w.blk_i + b);
  int boff;  // the block's offset: the sum of the earlier blocks' totals
  block_excl(pre, boff, sm.warp_tmp);
  if (b == G - 1 && t == 0) *total = boff + tot;
  int run = boff + woff;
  // (a warp whose range keeps nothing has nothing to write)
  for (long long base = wlo; cnt > 0 && base < whi; base += kCG) {
    int32_t v[kCU];
#pragma unroll
    for (int j = 0; j < kCU; ++j) {
      const long long i = base + j * 32 + lane;
      v[j] = i < whi ? __ldcg(in + i) : -1;
    }
#pragma unroll
    for (int j = 0; j < kCU; ++j) {
      const bool k = v[j] >= 0 && !bit_get(drop, v[j]);
      const unsigned mask = __ballot_sync(kFull, k);
      if (k) {
        out[run + __popc(mask & lanemask_lt())] = v[j];
        ty.list++;
      }
      run += __popc(mask);
    }
  }
  return true;
}

// ------------------------------------------------------------------------
// Trim phase: labels, valid bitmap, valid list (ordered), pivot, m_cand.
// SCC: a vertex with no out- or no in-edge is its own component
// (scc_trim, scc_trim.cpp:101-126); level 2 iterates to the fixed point with
// live degree counters.  WCC: a vertex with no edge at all (cc_trim.cpp:59-
// 84).  Pivot: SCC lowest id maximising out*in (> 0) (scc_main.cpp:169-182);
// WCC lowest id of maximum degree in the mirrored graph (cc_main.cpp:148-160).
// ------------------------------------------------------------------------
__device__ __forceinline__ bool better(unsigned long long k2, int32_t v2, unsigned long long k,
                                       int32_t v) {
  return k2 > k || (k2 == k && v2 >= 0 && (v < 0 || v2 < v));
}

// Ordered valid list: a warp's group of words with at least this many valid
// ids is written word by word by the whole warp; sparser groups go through
// the warp's staging buffer (which holds kWarpSmem >= this ids).
constexpr int kTrimDenseIds = 256;
static_assert(kTrimDenseIds <= kWarpSmem, "sparse groups fit the staging buffer");

// Size-2 components (an extension of the trim): u and p form a component
// when each is the other's only valid in-neighbour, or each the other's only
// valid out-neighbour (self-loops ignored).  Then nothing outside the pair
// reaches it (or is reached from it), and u and p reach each other.  Edges
// to vertices outside the valid set, and to vertices that other pairs
// remove during the same pass, come from or lead to whole components of
// their own, so they change no verdict.  Only vertices of degree at most
// kPairDeg in the tested direction are examined.
constexpr long long kPairDeg = 16;
__device__ __forceinline__ int32_t sole_valid_nbr(const Csr& cs, const uint32_t* valid, int32_t u) {
  const long long s = __ldg(cs.off + u), e = __ldg(cs.off + u + 1);
  if (e - s > kPairDeg) return -1;
  int32_t p = -1;
  for (long long i = s; i < e; ++i) {
    const int32_t x = __ldg(cs.adj + i);
    if (x == u || !bit_get(valid, x)) continue;
    if (p < 0) p = x;
    else if (x != p) return -1;
  }
  return p;
}
// The partner of u in a size-2 component when it has the larger id (the
// smaller member removes the pair), else -1.
__device__ __forceinline__ int32_t pair_partner(const GraphView& g, const uint32_t* valid,
                                                int32_t u) {
  int32_t p = sole_valid_nbr(g.in, valid, u);
  if (p > u && sole_valid_nbr(g.in, valid, p) == u) return p;
  p = sole_valid_nbr(g.out, valid, u);
  if (p > u && sole_valid_nbr(g.out, valid, p) == u) return p;
  return -1;
}

__device__ __forceinline__ void trim_phase(Args& A, Smem& sm) {
  Work& w = A.w;
  Ctl* c = w.ctl;
  const GraphView& g = A.g;
  const int G = gridDim.x, b = blockIdx.x, T = blockDim.x, t = threadIdx.x;
  const int warp = t >> 5, lane = t & 31;
  const bool scc = A.kind == kSCC;
  const bool level0 = scc && A.p.trim_level <= 0;
  const bool level2 = scc && A.p.trim_level >= 2;
  const bool pairs = scc && A.p.trim_pairs != 0;
  Tally ty;
  if (ld_vol(&c->err)) return;
  Steps st = steps_open(c);
  trace_rec(c, g.n, 16);
  // the FW-BW minima are folded with atomicMin later (read after this
  // kernel ends)
  if (b == 0 && t == 0) {
    c->minv[0] = 0x7fffffff;
    c->minv[1] = 0x7fffffff;
  }

  // Pass 1: warp k of the grid takes the 32-vertex word k.
  unsigned long long best_key = 0ull;  // out*in (SCC) or degree (WCC)
  int32_t best_v = -1;
  unsigned long long mc = 0ull;
  int removed = 0;
  const TrimVisit tv{w.vbits, w.live_in, w.live_out, w.label};
  Stage rs = stage_make(sm.stage(warp, 0));
  Out ro;
  ro.arr = w.x0;
  ro.base = 0;
  ro.cap = g.n;
  ro.counter = &step_out(c, st.s)->count;
  ro.edges = nullptr;
  ro.minv = nullptr;
  ro.where = 103;
  // Block b owns the contiguous word range [wlo, whi) (ranges in block
  // order, so the ordered valid list can be written per block); inside it
  // the warps take kTrimU consecutive words at a time, interleaved, and
  // issue all their offset loads before using any.  Each warp counts the
  // valid vertices it saw.
  constexpr int kTrimU = 4;
  // (a multiple of 4 words, so the list pass can read 16-byte groups)
  const long long bchunk = (((long long)w.nwords + G - 1) / G + 3) & ~3ll;
  const long long wlo = bchunk * b < w.nwords ? bchunk * b : w.nwords;
  const long long whi = wlo + bchunk < w.nwords ? wlo + bchunk : w.nwords;
  int wvalid = 0;  // warp-uniform
  // (a bulk L2 prefetch of the warp's next words, two iterations ahead, was
  // measured 3 us slower per R-MAT-24 run than none)
  const bool has_in = g.in.off != nullptr;
  for (long long wd0 = wlo + warp * kTrimU; wd0 < whi; wd0 += (T >> 5) * kTrimU) {
    long long o0[kTrimU], o1[kTrimU], i0[kTrimU], i1[kTrimU];
#pragma unroll
    for (int j = 0; j < kTrimU; ++j) {
      const long long vv = (wd0 + j) * 32 + lane;
      o0[j] = o1[j] = i0[j] = i1[j] = 0;
      if (wd0 + j < whi && vv < g.n) {
        o0[j] = __ldg(g.out.off + vv);
        o1[j] = __ldg(g.out.off + vv + 1);
        if (has_in) {
          i0[j] = __ldg(g.in.off + vv);
          i1[j] = __ldg(g.in.off + vv + 1);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < kTrimU; ++j) {
      const long long wd = wd0 + j;
      const long long vv = wd * 32 + lane;
      bool keep = false, gone = false;
      unsigned long long score = 0ull;
      if (wd < whi && vv < g.n) {
        const int32_t v = (int32_t)vv;
        const long long dout = o1[j] - o0[j];
        const long long din = i1[j] - i0[j];
        ty.vtx += g.in.off != nullptr ? 2 : 1;
        if (scc) {
          keep = level0 || (dout > 0 && din > 0);
          if (keep) {
            const unsigned long long prod = (unsigned long long)dout * (unsigned long long)din;
            if (prod > best_key) { best_key = prod; best_v = v; }
            mc += (unsigned long long)dout;
            score = prod;
          }
        } else {
          const long long deg = dout + din;
          keep = deg > 0;
          if (keep) {
            if ((unsigned long long)deg > best_key) { best_key = (unsigned long long)deg; best_v = v; }
            mc += (unsigned long long)deg;
            score = (unsigned long long)deg;
          }
        }
        gone = !keep;
        w.label[v] = keep ? -1 : v;
        if (level2) {
          w.live_out[v] = (int32_t)(dout < 0x7fffffffll ? dout : 0x7fffffffll);
          w.live_in[v] = (int32_t)(din < 0x7fffffffll ? din : 0x7fffffffll);
        }
        if (gone) ++removed;
      }
      const unsigned bits = __ballot_sync(kFull, keep);
      if (wd < whi && lane == 0) w.vbits[wd] = bits;
      wvalid += __popc(bits);
      if (level2) stage_push(rs, gone, (int32_t)vv, 0ull, ro, c);
      // batch: per-graph pivot, the packed key (score, lowest id) is maxed
      if (g.batch.gid != nullptr) {
        const unsigned long long mask = (1ull << g.batch.id_bits) - 1ull;
        const unsigned long long key =
            score ? ((score << g.batch.id_bits) | (mask - (unsigned long long)vv)) : 0ull;
        const int32_t gg = (wd < whi && vv < g.n) ? __ldg(g.batch.gid + vv) : -1;
        const int32_t g0 = __shfl_sync(kFull, gg, 0);
        if (__all_sync(kFull, gg == g0)) {
          unsigned long long kmax = key;
          for (int o = 16; o; o >>= 1) {
            const unsigned long long k2 = __shfl_xor_sync(kFull, kmax, o);
            kmax = k2 > kmax ? k2 : kmax;
          }
          if (lane == 0 && kmax && kmax > __ldcg(g.batch.pkey + g0)) atomicMax(g.batch.pkey + g0, kmax);
        } else if (key && gg >= 0 && key > __ldcg(g.batch.pkey + gg)) {
          atomicMax(g.batch.pkey + gg, key);
        }
      }
    }
  }
  if (level2) stage_flush(rs, ro, c);
  // Valid-list layout: block b writes the valid vertices of its word range
  // after those of the earlier blocks (blk_i[0, b)).
  int btot = 0;
  auto block_total = [&]() {
    __syncthreads();
    if (lane == 0) sm.warp_tmp[warp] = wvalid;
    __syncthreads();
    if (t == 0) {
      int s2 = 0;
      for (int i = 0; i < (T >> 5); ++i) s2 += sm.warp_tmp[i];
      sm.warp_tmp[kWarps] = s2;
      w.blk_i[b] = s2;
    }
    __syncthreads();
    btot = sm.warp_tmp[kWarps];
  };
  if (!level2 && !pairs) block_total();
  // block reduction of the pivot candidates
  {
    unsigned long long k = best_key;
    int32_t v = best_v;
    for (int o = 16; o; o >>= 1) {
      const unsigned long long k2 = __shfl_xor_sync(kFull, k, o);
      const int32_t v2 = __shfl_xor_sync(kFull, v, o);
      if (better(k2, v2, k, v)) { k = k2; v = v2; }
    }
    if (lane == 0) { sm.red_l[warp] = (long long)k; sm.red_i[warp] = v; }
    const unsigned long long msum = warp_sum64(mc);
    int rsum = removed;
    for (int o = 16; o; o >>= 1) rsum += __shfl_xor_sync(kFull, rsum, o);
    if (lane == 0) {
      if (msum) atomicAdd(&c->m_cand, msum);
      if (rsum) atomicAdd(&c->ntrim, rsum);
    }
    __syncthreads();
    if (t == 0) {
      unsigned long long bk = 0ull;
      int32_t bv = -1;
      for (int i = 0; i < kWarps; ++i) {
        if (better((unsigned long long)sm.red_l[i], sm.red_i[i], bk, bv)) {
          bk = (unsigned long long)sm.red_l[i];
          bv = sm.red_i[i];
        }
      }
      // the second half of blk_i: the first half holds the list counts
      w.blk_l[b] = (long long)bk;
      w.blk_i[G + b] = bv;
    }
  }
  if (!step_sync(c, st, 1)) return;
  trace_rec(c, 0, 17);
  if (b == 0 && warp == 0) {
    unsigned long long bk = 0ull;
    int32_t bv = -1;
    for (int i = lane; i < G; i += 32) {
      const unsigned long long k2 = (unsigned long long)__ldcg(w.blk_l + i);
      const int32_t v2 = __ldcg(w.blk_i + G + i);
      if (better(k2, v2, bk, bv)) { bk = k2; bv = v2; }
    }
    for (int o = 16; o; o >>= 1) {
      const unsigned long long k2 = __shfl_xor_sync(kFull, bk, o);
      const int32_t v2 = __shfl_xor_sync(kFull, bv, o);
      if (better(k2, v2, bk, bv)) { bk = k2; bv = v2; }
    }
    if (lane == 0) c->pivot = bk > 0ull ? bv : -1;
  }

  // Level 2: propagate removals to the fixed point.
  if (level2) {
    const Adj both = adj2(g.out, g.in);
    int32_t* bufs[2] = {w.x0, w.x1};
    int cur = 0;
    for (;;) {
      if (st.s - st.s0 >= A.p.tune.max_steps) { set_err(c, kErrIterLimit, 2); return; }
      const StepIn in = step_read(c, st.s);
      if (in.count == 0) break;
      const Sink sk = sink_make(bufs[cur ^ 1], 0, g.n, step_out(c, st.s), false, nullptr, nullptr,
                                0, 104);
      expand<2>(bufs[cur], in.count, nullptr, 0, both, tv, sk, A.p.tune, sm, c, ty);
      stat_inc(c, kStTrimSteps);
      if (!step_sync(c, st, 3)) return;
      cur ^= 1;
    }
  }
  // Size-2 components: warp k of the block takes the block's words k, k+32,
  // ...; each lane tests the vertex of its bit.
  if (pairs) {
    for (long long wd = wlo + warp; wd < whi; wd += (T >> 5)) {
      const uint32_t x = __ldcg(w.vbits + wd);  // one load: the same word in every lane
      if (x == 0u) continue;
      if ((x >> lane) & 1u) {
        const int32_t u = (int32_t)(wd * 32 + lane);
        const int32_t p = pair_partner(g, w.vbits, u);
        if (p >= 0 && bit_release(w.vbits, u)) {
          bit_release(w.vbits, p);
          w.label[u] = u;
          w.label[p] = u;
        }
      }
    }
    if (!step_sync(c, st, 7)) return;
  }
  // count the warp's share of the block's range again
  if (level2 || pairs) {
    wvalid = 0;
    for (long long wd0 = wlo + warp * 32; wd0 < whi; wd0 += (long long)T) {
      const long long wd = wd0 + lane;
      int x = wd < whi ? __popc(__ldcg(w.vbits + wd)) : 0;
      for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(kFull, x, o);
      wvalid += x;
    }
    block_total();
    if (!step_sync(c, st, 4)) return;
  }
  trace_rec(c, 0, 18);

  // Ordered valid list: per iteration each thread takes kListW consecutive
  // words (warp k of the block the k-th group of 32 x kListW); the warps'
  // counts are scanned in shared memory and each warp writes the ids of its
  // words.  The words are loaded before the block's offset is known.
  {
    constexpr int kListW = 4;
    const long long span = (long long)T * kListW;
    unsigned x[kListW];
    auto load_words = [&](long long base) {
      const long long wq = base + (long long)t * kListW;
      if (wq + kListW <= whi && (reinterpret_cast<uintptr_t>(w.vbits + wq) & 15u) == 0u) {
        const uint4 q4 = __ldcg(reinterpret_cast<const uint4*>(w.vbits + wq));
        x[0] = q4.x;
        x[1] = q4.y;
        x[2] = q4.z;
        x[3] = q4.w;
      } else {
#pragma unroll
        for (int j = 0; j < kListW; ++j) x[j] = wq + j < whi ? __ldcg(w.vbits + wq + j) : 0u;
      }
    };
    if (wlo < whi) load_words(wlo);
    int pre = 0;
    for (int j = t; j < b; j += T) pre += __ldcg(w.blk_i + j);
    int boff;
    block_excl(pre, boff, sm.warp_tmp);
    if (b == G - 1 && t == 0) {
      c->nvalid = boff + btot;
      if (level2 || pairs) c->ntrim = g.n - (boff + btot);
    }
    long long run = boff;
    for (long long base = wlo; base < whi; base += span) {
      if (base != wlo) load_words(base);
      const long long wq = base + (long long)t * kListW;
      int cs[kListW];
      int sum = 0;
#pragma unroll
      for (int j = 0; j < kListW; ++j) {
        cs[j] = sum;
        sum += __popc(x[j]);
      }
      int tot;
      const int ex = warp_excl(sum, tot);
      if (lane == 0) sm.warp_tmp[warp] = tot;
      __syncthreads();
      if (warp == 0) {
        const int y = lane < (T >> 5) ? sm.warp_tmp[lane] : 0;
        int incl = y;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const int z = __shfl_up_sync(kFull, incl, d);
          if (lane >= d) incl += z;
        }
        if (lane < (T >> 5)) sm.warp_tmp[lane] = incl - y;
        if (lane == 31) sm.warp_tmp[kWarps] = incl;
      }
      __syncthreads();
      const long long o = run + sm.warp_tmp[warp];
      run += sm.warp_tmp[kWarps];
      if (tot >= kTrimDenseIds) {
        // dense group: the warp writes its words one at a time, a lane per
        // bit, so every store is a contiguous run of ids
        const long long v0 = (base + (long long)warp * 32 * kListW) * 32;
#pragma unroll
        for (int j = 0; j < kListW; ++j) {
          unsigned nz = __ballot_sync(kFull, x[j] != 0u);
          while (nz) {
            const int k = __ffs(nz) - 1;
            nz &= nz - 1;
            const unsigned xk = __shfl_sync(kFull, x[j], k);
            const int ek = __shfl_sync(kFull, ex + cs[j], k);
            if ((xk >> lane) & 1u)
              w.listA[o + ek + __popc(xk & ((1u << lane) - 1u))] =
                  (int32_t)(v0 + (long long)(k * kListW + j) * 32 + lane);
          }
        }
      } else {
        // sparse group: each lane puts its words' ids at their ranks in the
        // warp's staging buffer (visiting each word's bits from bit `lane`
        // on, so that the lanes of dense words hit different banks), then
        // the warp copies the buffer out
        int32_t* buf = sm.stage(warp, 0);
#pragma unroll
        for (int j = 0; j < kListW; ++j) {
          const unsigned xj = x[j];
          unsigned y = (xj >> lane) | (lane ? xj << (32 - lane) : 0u);
          while (y) {
            const int p = __ffs(y) - 1;
            y &= y - 1;
            const int bit = (p + lane) & 31;
            buf[ex + cs[j] + __popc(xj & ((1u << bit) - 1u))] = (int32_t)((wq + j) * 32 + bit);
          }
        }
        __syncwarp();
        for (int k = lane; k < tot; k += 32) w.listA[o + k] = buf[k];
        __syncwarp();
      }
      ty.list += sum;
      __syncthreads();
    }
  }
  if (!step_sync(c, st, 5)) return;
  trace_rec(c, 0, 19);
  // A hint replaces the pivot; level 2 may have trimmed the pivot, in which
  // case FW-BW is skipped and the colour rounds label what is left.
  if (b == 0 && t == 0) {
    int32_t pv = c->pivot;
    if (A.p.pivot_hint >= 0 && A.p.pivot_hint < g.n) pv = A.p.pivot_hint;
    if (pv >= 0 && !bit_get(w.vbits, pv)) pv = -1;
    c->pivot = pv;
  }
  // batch: every graph's pivot that survived trim is a root
  if (g.batch.gid != nullptr) {
    const unsigned long long mask = (1ull << g.batch.id_bits) - 1ull;
    for (long long gi0 = (long long)b * T; gi0 < g.batch.count; gi0 += (long long)G * T) {
      const long long gi = gi0 + t;
      int32_t v = -1;
      if (gi < g.batch.count) {
        const unsigned long long key = __ldcg(g.batch.pkey + gi);
        if (key) {
          v = (int32_t)(mask - (key & mask));
          if (!bit_get(w.vbits, v)) v = -1;
        }
      }
      list_append(v >= 0, v, g.batch.roots, &c->nroots, g.batch.count, c, 6);
    }
  }
  tally_flush(ty, c, kKTrim, A.p.count_unassigned != 0, sm.red_u);
  steps_close(c, st);
}

// ------------------------------------------------------------------------
// Direction-optimising reachability from `root`, run by the whole grid.
// Push steps expand the frontier (the vertices appended by the previous
// step) with ReachVisit; pull steps let every unreached candidate scan its
// pull adjacency for a reached vertex and stop at the first
// (scc_fwbw.cpp:116-149).  Push -> pull when the frontier's edge count times
// alpha exceeds the unvisited edge estimate; pull -> push when the frontier
// has fewer than ncand / beta vertices.  q receives every reached vertex
// exactly once, so q[0, result) is the reached set; *minv gets its smallest
// id.  Returns -1 on error.
// ------------------------------------------------------------------------
struct ReachSpec {
  bool local;             // push steps may run local rounds (its visit list is not
                          // read afterwards, and its graph is sparse)
  Adj push, pull;
  const uint32_t* allow;
  uint32_t* vis;
  const int32_t* cand;
  int32_t ncand;
  unsigned long long m_cand;
  const int32_t* roots;   // sources (distinct, allowed)
  int32_t nroots;
  int32_t* q;
  int32_t* minv;
  int stat_slot;
};

constexpr int kPullU = 4;  // backlog candidates per thread per edge pass
constexpr int kPullA = 8;  // candidates per thread per hint pass

// One pull step: every unreached candidate looks for a reached
// pull-neighbour (scc_fwbw.cpp:116-149, which scans until the first hit).
// Three tiers keep the work balanced:
//   thread: a hint pass over kPullA candidates per thread (its loads do not
//           depend on one another beyond the candidate id), then, for the
//           candidates the hint did not settle, an edge pass of up to
//           kPullThread edges, kPullU candidates per thread, run whenever a
//           warp's backlog holds 32 * kPullU of them;
//   warp  : candidates with more edges, one warp each, 32 * kPullWU edges
//           per iteration, up to kPullWarpEdges edges;
//   block : the rest, one block each, kBlock edges per iteration.
// The warp and block tiers run after a grid barrier on lists the thread
// tier filled, spread over the whole grid.  Found candidates are appended
// to q; candidates with no reached neighbour are kept in cand_next.
constexpr int kPullThread = 4;
constexpr long long kPullWarpEdges = 1024;
constexpr int kPullWU = 4;  // warp tier: edges per lane per iteration
static_assert(kTodo >= 32 * kPullU - 1 + 32 * kPullA, "pull backlog too small");

// Edge pass of the pull thread tier over todo[0, cnt) (cnt <= 32 * kPullU;
// warp-uniform; every candidate is unreached and not settled by its hint).
template <int NC>
__device__ __forceinline__ void pull_edges(const ReachSpec& R, const int32_t* todo, int cnt,
                                           int kt, Stage& sf, Stage& sk, const Out& of,
                                           const Out& ok, int32_t* wl, int32_t* bl, int32_t* lc,
                                           int32_t n, Ctl* c, Tally& ty) {
  const int lane = lane_id();
  int32_t v[kPullU];
  bool found[kPullU];
  long long s0[kPullU], d0[kPullU], s1[kPullU], d1[kPullU];
  int32_t u[kPullU][kPullThread];
#pragma unroll
  for (int j = 0; j < kPullU; ++j) {
    const int i = j * 32 + lane;
    v[j] = i < cnt ? todo[i] : -1;
  }
#pragma unroll
  for (int j = 0; j < kPullU; ++j) {
    s0[j] = d0[j] = s1[j] = d1[j] = 0;
    if (v[j] >= 0) {
      rec_load<NC>(R.pull, v[j], s0[j], d0[j], s1[j], d1[j]);
      ty.vtx += NC;
    }
  }
  // the first kt edges of every candidate, loads overlapped
#pragma unroll
  for (int j = 0; j < kPullU; ++j) {
#pragma unroll
    for (int e = 0; e < kPullThread; ++e) {
      u[j][e] = -1;
      if (v[j] >= 0 && e < kt && e < d0[j] + d1[j]) {
        int k;
        u[j][e] = adj_at<NC>(R.pull, s0[j], d0[j], s1[j], e, k);
      }
    }
  }
  bool to_warp[kPullU], to_block[kPullU], keep[kPullU];
#pragma unroll
  for (int j = 0; j < kPullU; ++j) {
    found[j] = false;
#pragma unroll
    for (int e = 0; e < kPullThread; ++e) {
      if (u[j][e] >= 0) {
        ty.edges++;
        if (!found[j] && bit_get_l1(R.vis, u[j][e])) found[j] = true;
      }
    }
    const long long d = d0[j] + d1[j];
    const bool open = v[j] >= 0 && !found[j];
    to_warp[j] = open && d > kt && d <= kt + kPullWarpEdges;
    to_block[j] = open && d > kt + kPullWarpEdges;
    keep[j] = open && d <= kt;
  }
#pragma unroll
  for (int j = 0; j < kPullU; ++j) {
    // a pull candidate has one owner: its bit is set without a reply
    if (found[j]) bit_set_red(R.vis, v[j]);
    stage_push(sf, found[j], v[j], 0ull, of, c);
    stage_push(sk, keep[j], v[j], 0ull, ok, c);
    list_append(to_warp[j], v[j], wl, &lc[0], n, c, 204);
    list_append(to_block[j], v[j], bl, &lc[1], n, c, 205);
  }
}

// The outputs of a pull step: found vertices to q (from qhi on), kept
// candidates to cand_next, with the counters of the search's slot.
__device__ __forceinline__ void pull_outs(const ReachSpec& R, const Work& w, int32_t* cand_next,
                                          long long qhi, Slot* o, Out& of, Out& ok) {
  of.arr = R.q;
  of.base = qhi;
  of.cap = w.n;
  of.counter = &o->count;
  of.edges = nullptr;
  of.minv = R.minv;
  of.where = 202;
  ok.arr = cand_next;
  ok.base = 0;
  ok.cap = w.n;
  ok.counter = &o->cand;
  ok.edges = nullptr;
  ok.minv = nullptr;
  ok.where = 203;
}

__device__ __forceinline__ int pull_kt(const Args& A) {
  return A.p.tune.k_pull < kPullThread ? (A.p.tune.k_pull > 0 ? A.p.tune.k_pull : 1) : kPullThread;
}

// Thread tier of a pull step (search `dir`, its pp-th pull step): fills the
// warp- and block-tier lists wl / bl; the caller's grid barrier then
// completes them for pull_tail.
template <int NC>
__device__ void pull_thread(const ReachSpec& R, const Args& A, Work& w, Smem& sm, Tally& ty,
                            const int32_t* cand_cur, int32_t ncur, int32_t* cand_next,
                            long long qhi, Slot* o, int pp, int dir, int32_t* wl, int32_t* bl) {
  Ctl* c = w.ctl;
  const int G = gridDim.x, b = blockIdx.x, T = blockDim.x, t = threadIdx.x;
  const int warp = t >> 5, lane = t & 31;
  int32_t* lc = c->lcount[dir][pp & 1];
  long long* pnext = &c->pnext[dir][pp & 1];
  if (b == 0 && t == 0) {
    c->lcount[dir][(pp + 1) & 1][0] = 0;
    c->lcount[dir][(pp + 1) & 1][1] = 0;
    c->pnext[dir][(pp + 1) & 1] = 0;
  }
  const int kt = pull_kt(A);
  Out of, ok;
  pull_outs(R, w, cand_next, qhi, o, of, ok);
  const unsigned long long edges0 = ty.edges;
  Stage sf = stage_make(sm.stage(warp, 0));
  Stage sk = stage_make(sm.stage(warp, 1));
  int32_t* todo = sm.todo(warp);
  int ntodo = 0;  // warp-uniform
  const long long nw = (long long)G * (T >> 5);
  const bool hints = R.pull.c[0].hint != nullptr;
  // warps claim runs of candidates from a shared counter, so a warp whose
  // candidates settle quickly takes more of them; a run is about a quarter
  // of a warp's even share (between 32 and 2 * kGroup)
  constexpr long long kGroup = 32 * kPullA;
  constexpr int kEdgeBatch = 32 * kPullU;
  long long grab = (long long)ncur / (nw * 4) / 32 * 32;
  grab = grab < 32 ? 32 : (grab > 2 * kGroup ? 2 * kGroup : grab);
  for (;;) {
    long long clo = 0;
    if (lane == 0)
      clo = (long long)atomicAdd((unsigned long long*)pnext, (unsigned long long)grab);
    clo = shfl64(clo, 0);
    if (clo >= ncur) break;
    const long long chi = clo + grab < ncur ? clo + grab : ncur;
    for (long long base = clo; base < chi; base += kGroup) {
      int32_t v[kPullA], h0[kPullA], h1[kPullA];
#pragma unroll
      for (int j = 0; j < kPullA; ++j) {
        const long long i = base + j * 32 + lane;
        v[j] = i < chi ? __ldcg(cand_cur + i) : -1;
      }
      // the hint (the neighbour of largest degree) settles most candidates
      // without touching the CSR; it is read before the candidate's own bit
      // is known so that the two loads overlap
#pragma unroll
      for (int j = 0; j < kPullA; ++j) {
        h0[j] = (v[j] >= 0 && hints) ? __ldg(R.pull.c[0].hint + v[j]) : -1;
        h1[j] = -1;
        if constexpr (NC > 1) {
          if (v[j] >= 0 && R.pull.c[1].hint != nullptr) h1[j] = __ldg(R.pull.c[1].hint + v[j]);
        }
      }
      bool unv[kPullA];
#pragma unroll
      for (int j = 0; j < kPullA; ++j) unv[j] = v[j] >= 0 && !bit_get_l1(R.vis, v[j]);
#pragma unroll
      for (int j = 0; j < kPullA; ++j) {
        const bool hinted = unv[j] && ((h0[j] >= 0 && bit_get_l1(R.vis, h0[j])) ||
                                       (h1[j] >= 0 && bit_get_l1(R.vis, h1[j])));
        if (v[j] >= 0) ty.list++;
        if (hinted) bit_set_red(R.vis, v[j]);
        stage_push(sf, hinted, v[j], 0ull, of, c);
        // the rest go to the warp's backlog
        const bool open = unv[j] && !hinted;
        const unsigned mask = __ballot_sync(kFull, open);
        if (open) todo[ntodo + __popc(mask & lanemask_lt())] = v[j];
        ntodo += __popc(mask);
      }
      __syncwarp();
      if (ntodo >= kEdgeBatch) {
        int done = 0;
        while (ntodo - done >= kEdgeBatch) {
          pull_edges<NC>(R, todo + done, kEdgeBatch, kt, sf, sk, of, ok, wl, bl, lc, w.n, c, ty);
          done += kEdgeBatch;
        }
        // move the remainder (< kEdgeBatch, from at or above kEdgeBatch) to the front
        __syncwarp();
        for (int i = lane; i < ntodo - done; i += 32) todo[i] = todo[done + i];
        __syncwarp();
        ntodo -= done;
      }
    }
  }
  if (ntodo > 0) pull_edges<NC>(R, todo, ntodo, kt, sf, sk, of, ok, wl, bl, lc, w.n, c, ty);
  if (pp == 0 && dir == 0 && t == 0 && b < kBlkTimes) c->blk_t[b] = gtimer();
  stage_flush(sf, of, c);
  stage_flush(sk, ok, c);
  ty.pull_edges += ty.edges - edges0;
}

// Warp and block tiers of a pull step, after the grid barrier that follows
// every search's thread tier.
template <int NC>
__device__ void pull_tail(const ReachSpec& R, const Args& A, Work& w, Smem& sm, Tally& ty,
                          int32_t* cand_next, long long qhi, Slot* o, int pp, int dir,
                          const int32_t* wl, const int32_t* bl) {
  Ctl* c = w.ctl;
  const int G = gridDim.x, b = blockIdx.x, T = blockDim.x, t = threadIdx.x;
  const int warp = t >> 5, lane = t & 31;
  const int32_t* lc = c->lcount[dir][pp & 1];
  const int kt = pull_kt(A);
  Out of, ok;
  pull_outs(R, w, cand_next, qhi, o, of, ok);
  const unsigned long long edges0 = ty.edges;
  Stage sf = stage_make(sm.stage(warp, 0));
  Stage sk = stage_make(sm.stage(warp, 1));
  const long long nw = (long long)G * (T >> 5);
  const int32_t nwl = __ldcg(&lc[0]), nbl = __ldcg(&lc[1]);
  for (long long j = (long long)b * (T >> 5) + warp; j < nwl; j += nw) {
    const int32_t v = __ldcg(wl + j);
    long long s0, d0, s1, d1;
    rec_load<NC>(R.pull, v, s0, d0, s1, d1);
    const long long d = d0 + d1;
    bool found = false;
    // kPullWU edges per lane per iteration, loads overlapped
    for (long long e0 = kt; e0 < d && !found; e0 += 32 * kPullWU) {
      int32_t x[kPullWU];
#pragma unroll
      for (int q = 0; q < kPullWU; ++q) {
        const long long e = e0 + q * 32 + lane;
        x[q] = -1;
        if (e < d) {
          int k;
          x[q] = adj_at<NC>(R.pull, s0, d0, s1, e, k);
        }
      }
      bool hit = false;
#pragma unroll
      for (int q = 0; q < kPullWU; ++q) {
        if (x[q] >= 0) {
          ty.edges++;
          hit = hit || bit_get_l1(R.vis, x[q]);
        }
      }
      found = __any_sync(kFull, hit);
    }
    if (found && lane == 0) bit_set_red(R.vis, v);
    stage_push(sf, found && lane == 0, v, 0ull, of, c);
    stage_push(sk, !found && lane == 0, v, 0ull, ok, c);
  }
  for (long long j = b; j < nbl; j += G) {
    const int32_t v = __ldcg(bl + j);
    long long s0, d0, s1, d1;
    rec_load<NC>(R.pull, v, s0, d0, s1, d1);
    const long long d = d0 + d1;
    bool found = false;
    for (long long e0 = kt; e0 < d; e0 += T) {
      const long long e = e0 + t;
      bool hit = false;
      if (e < d) {
        int k;
        const int32_t x = adj_at<NC>(R.pull, s0, d0, s1, e, k);
        ty.edges++;
        hit = bit_get_l1(R.vis, x);
      }
      if (__syncthreads_or(hit)) {
        found = true;
        break;
      }
    }
    if (warp == 0) {
      if (found && lane == 0) bit_set_red(R.vis, v);
      stage_push(sf, found && lane == 0, v, 0ull, of, c);
      stage_push(sk, !found && lane == 0, v, 0ull, ok, c);
    }
  }
  stage_flush(sf, of, c);
  stage_flush(sk, ok, c);
  ty.pull_edges += ty.edges - edges0;
}

// Pivot degree (smaller of in and out) from which the two searches of an
// SCC run in the same steps.
constexpr long long kTogetherDegree = 64;
// Average push degree of the valid vertices up to which searches run local
// rounds in their push steps.
constexpr double kLocalAvgDegree = 8.0;

// One search (one direction of one traversal): its spec, the lists it owns,
// and its running state.
struct Search {
  ReachSpec R;
  int dir;                 // its counter set in the step ring and pull claims
  int32_t* cand[2];        // pull candidate lists (alternating)
  int32_t* heavy[2];       // push heavy-vertex lists (alternating)
  int32_t* wl;             // pull warp-tier list
  int32_t* bl;             // pull block-tier list
  long long qlo, qhi;      // this step's frontier: q[qlo, qhi)
  long long remaining;     // unreached candidates (estimate after push steps)
  double avg;              // average push degree of the candidates
  const int32_t* cand_cur;
  int32_t ncur;
  int32_t huge;            // heavy vertices deferred into this step
  int cn;                  // cand[cn] receives the next kept list
  int hsel;
  int pp;                  // pull steps so far
  int ti;                  // this step's trace record, or -1
  bool pull, prev_pull, active;
};

// Runs the searches S[0, ns) to completion, all advancing in the same steps:
// in each step every active search pushes its frontier or runs a pull step;
// the pull steps share one internal grid barrier between their thread tiers
// and their warp / block tiers.  S and flags are in shared memory: thread 0
// updates them (every block computes the same state from the same
// counters) and the block barrier that follows publishes them.  Returns
// false when the kernel must stop.
// kOptions: the optional run features are compiled in (here the edge-
// balanced push, Tune::expand_mode 1).
template <int NC, bool kOptions = false>
__device__ bool reach_multi(Search* S, int ns, int* flags /* shared, 2 */, const Args& A,
                            Work& w, Smem& sm, Steps& st, Tally& ty) {
  Ctl* c = w.ctl;
  const int G = gridDim.x, b = blockIdx.x, T = blockDim.x, t = threadIdx.x;
  const int warp = t >> 5, lane = t & 31;
  const Tune& tn = A.p.tune;
  // the sources are the first step's frontier
  for (int k = 0; k < ns; ++k) {
    const ReachSpec& R = S[k].R;
    Out ro;
    ro.arr = R.q;
    ro.base = 0;
    ro.cap = w.n;
    ro.counter = &step_out(c, st.s, S[k].dir)->count;
    ro.edges = &step_out(c, st.s, S[k].dir)->edges;
    ro.minv = R.minv;
    ro.where = 207;
    Stage rs = stage_make(sm.stage(warp, 0));
    for (long long base = (long long)b * T + (t & ~31); base < R.nroots;
         base += (long long)G * T) {
      const long long i = base + lane;
      bool take = false;
      int32_t r = 0;
      if (i < R.nroots) {
        r = __ldcg(R.roots + i);
        take = bit_claim(R.vis, r);
      }
      stage_push(rs, take, r, take ? adj_degree<NC>(R.push, r) : 0ull, ro, c);
    }
    stage_flush(rs, ro, c);
  }
  if (t == 0) {
    for (int k = 0; k < ns; ++k) {
      Search& q = S[k];
      q.qlo = q.qhi = 0;
      q.remaining = q.R.ncand;
      q.avg = q.R.ncand > 0 ? (double)q.R.m_cand / (double)q.R.ncand : 0.0;
      q.cand_cur = q.R.cand;
      q.ncur = q.R.ncand;
      q.cn = 0;
      q.hsel = 0;
      q.pp = 0;
      q.pull = q.prev_pull = false;
      q.active = true;
    }
  }
  if (!step_sync(c, st, 20)) return false;
  const int s_start = st.s;
  for (;;) {
    if (st.s - s_start >= tn.max_steps) { set_err(c, kErrIterLimit, 21); return false; }
    if (t == 0) {
      int nactive = 0, any_pull = 0;
      for (int k = 0; k < ns; ++k) {
        Search& q = S[k];
        q.ti = -1;
        if (!q.active) continue;
        const StepIn in = step_read(c, st.s, q.dir);
        q.qlo = q.qhi;
        q.qhi = q.qlo + in.count;
        q.huge = in.huge;
        // a pull step does not read the push degrees of what it finds; its
        // frontier edge count is estimated from the average degree
        const unsigned long long medges =
            q.prev_pull ? (unsigned long long)((double)in.count * q.avg) : in.edges;
        if (q.prev_pull) {
          q.cand_cur = q.cand[q.cn];
          q.ncur = in.cand;
          q.cn ^= 1;
          q.remaining = in.cand;
        } else {
          q.remaining = q.remaining > in.count ? q.remaining - in.count : 0;
        }
        // push -> pull when the frontier's edges outweigh the unexplored
        // edges (estimated from the unreached candidates); pull -> push when
        // the frontier is small against the candidates
        if (!q.pull) {
          const double mu = (double)q.remaining * q.avg;
          if ((double)medges * (double)tn.alpha > mu) q.pull = true;
        } else if ((double)in.count * (double)tn.beta < (double)q.R.ncand) {
          q.pull = false;
        }
        if (b == 0) {
          q.ti = c->ntrace % kTrace;
          c->trace[q.ti].t = gtimer();
          c->trace[q.ti].t_mid = 0;
          c->trace[q.ti].nwarp = 0;
          c->trace[q.ti].nblock = 0;
          c->trace[q.ti].count = in.count;
          c->trace[q.ti].mode =
              (q.pull ? 1 : 0) | (in.huge > 0 ? 2 : 0) | (q.R.stat_slot == kStBwSteps ? 4 : 0);
          c->ntrace++;
        }
        if (in.count == 0 && (q.pull || in.huge == 0)) {
          q.active = false;
          continue;
        }
        ++nactive;
        any_pull |= q.pull ? 1 : 0;
      }
      flags[0] = nactive;
      flags[1] = any_pull;
    }
    __syncthreads();
    if (flags[0] == 0) break;
    const bool any_pull = flags[1] != 0;
    for (int k = 0; k < ns; ++k) {
      const Search& q = S[k];
      if (!q.active) continue;
      Slot* o = step_out(c, st.s, q.dir);
      if (!q.pull) {
        const ReachVisit<NC> rv{q.R.allow, q.R.vis, q.R.push, q.R.local};
        const Sink sk = sink_make(q.R.q, q.qhi, w.n, o, true, q.R.minv, q.heavy[q.hsel ^ 1], w.n,
                                  201);
        bool tiers = true;
        if constexpr (kOptions) {
          if (tn.expand_mode == 1) {
            // (its group prefixes go to the search's pull warp-tier list and
            // its block totals to the search's half of blk_l, both free in
            // a push step)
            if (!expand_balanced<NC>(q.R.q + q.qlo, (int32_t)(q.qhi - q.qlo), q.R.push, rv, sk,
                                     reinterpret_cast<long long*>(q.wl),
                                     w.blk_l + (long long)q.dir * G, sm, c, ty))
              return false;
            tiers = false;
          }
        }
        if (tiers)
          expand<NC>(q.R.q + q.qlo, (int32_t)(q.qhi - q.qlo), q.heavy[q.hsel], q.huge, q.R.push,
                     rv, sk, tn, sm, c, ty);
      } else {
        pull_thread<NC>(q.R, A, w, sm, ty, q.cand_cur, q.ncur, q.cand[q.cn], q.qhi, o, q.pp,
                        q.dir, q.wl, q.bl);
      }
    }
    if (any_pull) {
      // the warp and block tiers need the complete lists
      if (!grid_barrier(c, 206)) return false;
      for (int k = 0; k < ns; ++k) {
        const Search& q = S[k];
        if (!q.active || !q.pull) continue;
        if (b == 0 && t == 0 && q.ti >= 0) {
          c->trace[q.ti].t_mid = gtimer();
          c->trace[q.ti].nwarp = __ldcg(&c->lcount[q.dir][q.pp & 1][0]);
          c->trace[q.ti].nblock = __ldcg(&c->lcount[q.dir][q.pp & 1][1]);
        }
        pull_tail<NC>(q.R, A, w, sm, ty, q.cand[q.cn], q.qhi, step_out(c, st.s, q.dir), q.pp,
                      q.dir, q.wl, q.bl);
      }
    }
    __syncthreads();
    if (t == 0) {
      for (int k = 0; k < ns; ++k) {
        Search& q = S[k];
        if (!q.active) continue;
        if (q.pull) {
          ++q.pp;
          stat_inc(c, kStPullSteps);
        }
        q.prev_pull = q.pull;
        stat_inc(c, q.R.stat_slot);
        q.hsel ^= 1;
      }
    }
    if (!step_sync(c, st, 24)) return false;
  }
  return true;
}

// ------------------------------------------------------------------------
// Re-pivot between FW-BW rounds (the reference runs one round): the next
// pivot is the valid vertex of largest out*in (SCC) or degree (WCC), lowest
// id on ties, found over the compacted valid list by the first round's rule;
// the candidates' edge count is summed alongside.  Also clears the visit
// bitmaps and minima for the next round.  Returns false when the kernel must
// stop.
// ------------------------------------------------------------------------
constexpr int32_t kRepivotMin = 4096;  // fewer valid vertices: no further round
__device__ bool repivot(const Args& A, Smem& sm) {
  const Work& w = A.w;
  Ctl* c = w.ctl;
  const GraphView& g = A.g;
  const int G = gridDim.x, b = blockIdx.x, T = blockDim.x, t = threadIdx.x;
  const int warp = t >> 5, lane = t & 31;
  const bool scc = A.kind == kSCC;
  // the last round's valid list, counters and step number are complete
  if (!grid_barrier(c, 29)) return false;
  Steps st = steps_open(c);
  const int32_t nv = __ldcg(&c->nvalid);
  unsigned long long bk = 0ull, msum = 0ull;
  int32_t bv = -1;
  for (long long i = (long long)b * T + t; i < nv; i += (long long)G * T) {
    const int32_t v = __ldcg(w.listA + i);
    const long long dout = __ldg(g.out.off + v + 1) - __ldg(g.out.off + v);
    const long long din = g.in.off != nullptr ? __ldg(g.in.off + v + 1) - __ldg(g.in.off + v) : 0;
    const unsigned long long key = scc ? (unsigned long long)dout * (unsigned long long)din
                                       : (unsigned long long)(dout + din);
    msum += scc ? (unsigned long long)dout : (unsigned long long)(dout + din);
    if (better(key, v, bk, bv)) { bk = key; bv = v; }
  }
  for (long long wd = (long long)b * T + t; wd < w.nwords; wd += (long long)G * T) {
    w.fvis[wd] = 0u;
    w.bvis[wd] = 0u;
  }
  for (int o = 16; o; o >>= 1) {
    const unsigned long long k2 = __shfl_xor_sync(kFull, bk, o);
    const int32_t v2 = __shfl_xor_sync(kFull, bv, o);
    if (better(k2, v2, bk, bv)) { bk = k2; bv = v2; }
  }
  msum = warp_sum64(msum);
  __syncthreads();
  if (lane == 0) {
    sm.red_l[warp] = (long long)bk;
    sm.red_i[warp] = bv;
    sm.red_u[warp] = msum;
  }
  __syncthreads();
  if (t == 0) {
    unsigned long long k = 0ull, ms = 0ull;
    int32_t v = -1;
    for (int i = 0; i < (T >> 5); ++i) {
      if (better((unsigned long long)sm.red_l[i], sm.red_i[i], k, v)) {
        k = (unsigned long long)sm.red_l[i];
        v = sm.red_i[i];
      }
      ms += sm.red_u[i];
    }
    w.blk_l[b] = (long long)k;
    w.blk_i[G + b] = v;
    w.blk_l[G + b] = (long long)ms;
  }
  if (!step_sync(c, st, 30)) return false;
  if (b == 0 && warp == 0) {
    unsigned long long k = 0ull, ms = 0ull;
    int32_t v = -1;
    for (int i = lane; i < G; i += 32) {
      const unsigned long long k2 = (unsigned long long)__ldcg(w.blk_l + i);
      const int32_t v2 = __ldcg(w.blk_i + G + i);
      if (better(k2, v2, k, v)) { k = k2; v = v2; }
      ms += (unsigned long long)__ldcg(w.blk_l + G + i);
    }
    for (int o = 16; o; o >>= 1) {
      const unsigned long long k2 = __shfl_xor_sync(kFull, k, o);
      const int32_t v2 = __shfl_xor_sync(kFull, v, o);
      if (better(k2, v2, k, v)) { k = k2; v = v2; }
    }
    ms = warp_sum64(ms);
    if (lane == 0) {
      c->rpivot = k > 0ull ? v : -1;
      c->m_cand = ms;
      c->minv[0] = 0x7fffffff;
      c->minv[1] = 0x7fffffff;
      if (k > 0ull) c->nrounds++;
    }
  }
  steps_close(c, st);
  // the new pivot, edge count, minima, cleared bitmaps and step number
  return grid_barrier(c, 31);
}

// ------------------------------------------------------------------------
// Reach phase: SCC -> forward and backward reachability from the pivot; the SCC
// (reached both ways) leaves the valid list labelled with its smallest id
// (or the pivot, with canonical labels off), as update_valid does with the
// pivot (scc_fwbw, scc_fwbw.cpp:412-513).  WCC -> one search over the union
// adjacency (cc_bfs, cc_bfs.cpp:217-291).
// ------------------------------------------------------------------------
// kRepeat: a round after the first, from the pivot chosen by repivot;
// kOptions: as for reach_multi.
template <int NC, bool kRepeat = false, bool kOptions = false>
__device__ __forceinline__ void reach_phase(Args& A, Smem& sm) {
  Work& w = A.w;
  Ctl* c = w.ctl;
  const GraphView& g = A.g;
  const int G = gridDim.x, b = blockIdx.x, T = blockDim.x, t = threadIdx.x;
  Tally ty;
  if (ld_vol(&c->err)) return;
  const bool batch = g.batch.gid != nullptr;
  int32_t* const pv = kRepeat ? &c->rpivot : &c->pivot;
  const int32_t pivot = __ldcg(pv);
  const int32_t nvalid = __ldcg(&c->nvalid);
  const int32_t* roots = batch ? g.batch.roots : pv;
  const int32_t nroots = batch ? __ldcg(&c->nroots) : (pivot >= 0 ? 1 : 0);
  if (nroots == 0 || nvalid == 0) return;
  Steps st = steps_open(c);
  const bool scc = A.kind == kSCC;
  const uint32_t* hit;
  int32_t* hit_min;
  ReachSpec F;
  F.push = scc ? adj1(g.out) : adj_undirected(g);
  F.pull = scc ? adj1(g.in) : F.push;
  F.allow = w.vbits;
  F.vis = w.fvis;
  F.cand = w.listA;
  F.ncand = nvalid;
  F.m_cand = __ldcg(&c->m_cand);
  F.roots = roots;
  F.nroots = nroots;
  F.q = w.q;
  F.minv = batch ? nullptr : &c->minv[0];
  F.stat_slot = kStFwSteps;
  // SCC of one graph from a hub pivot: both searches run in the same steps,
  // the backward one over the whole valid set, and the component is what
  // both reach.  Otherwise (a low-degree pivot, where the backward set can
  // be far larger than the forward one; batches) the backward search runs
  // after the forward one, inside the forward set, as the reference does.
  bool together = false;
  if constexpr (NC == 1) {
    if (scc && !batch) {
      const long long dout = g.out.off[pivot + 1] - g.out.off[pivot];
      const long long din = g.in.off[pivot + 1] - g.in.off[pivot];
      together = (dout < din ? dout : din) >= kTogetherDegree;
    }
  }
  // Local rounds in push steps: on sparse graphs, and only for a search
  // whose visit list is not read afterwards (the forward list of a
  // sequential SCC is the backward search's candidate list).
  const bool sparse = (double)F.m_cand <= kLocalAvgDegree * (double)nvalid;
  F.local = sparse && (!scc || together);
  // the search states live in shared memory (one copy per block, written
  // by thread 0), not in every thread's local memory
  __shared__ Search srch[2];
  __shared__ int sflags[2];
  Search& SF = srch[0];
  Search& SB = srch[1];
  if (t == 0) {
    SF.R = F;
    SF.dir = 0;
    SF.cand[0] = w.candA;
    SF.cand[1] = w.candB;
    SF.heavy[0] = w.h0;
    SF.heavy[1] = w.h1;
    SF.wl = w.x1;
    SF.bl = w.h1;
    // the backward search's lists are all its own (live-degree counters,
    // colours and the second valid list are free until the later phases)
    SB.dir = 1;
    SB.cand[0] = w.live_in;
    SB.cand[1] = w.live_out;
    SB.heavy[0] = w.colour;
    SB.heavy[1] = w.listB;
    SB.wl = w.xa;
    SB.bl = w.xb;
  }
  ReachSpec B;
  B.push = adj1(g.in);
  B.pull = adj1(g.out);
  B.m_cand = F.m_cand;
  B.roots = roots;
  B.nroots = nroots;
  B.q = w.x0;
  B.stat_slot = kStBwSteps;
  B.local = sparse;
  if constexpr (NC == 1) {
    if (together) {
      B.allow = w.vbits;
      B.vis = w.bvis;
      B.cand = w.listA;
      B.ncand = nvalid;
      B.minv = nullptr;
      if (t == 0) SB.R = B;
      __syncthreads();
      if (!reach_multi<NC, kOptions>(srch, 2, sflags, A, w, sm, st, ty)) return;
      // the component is what both searches reached: its smallest member,
      // while the backward bitmap becomes the intersection (the forward
      // count comes from the bitmap: local rounds leave no visit list)
      int32_t mn = 0x7fffffff;
      int nfw = 0;
      for (long long wd = (long long)b * T + t; wd < w.nwords; wd += (long long)G * T) {
        const uint32_t bw = __ldcg(w.bvis + wd);
        const uint32_t fw = __ldcg(w.fvis + wd);
        const uint32_t x = fw & bw;
        if (x != bw) w.bvis[wd] = x;
        nfw += __popc(fw);
        if (x) {
          const int32_t v0 = (int32_t)(wd * 32 + __ffs(x) - 1);
          mn = v0 < mn ? v0 : mn;
        }
      }
      mn = warp_min(mn);
      for (int o = 16; o; o >>= 1) nfw += __shfl_xor_sync(kFull, nfw, o);
      if (lane_id() == 0) {
        if (mn != 0x7fffffff) atomicMin(&c->minv[1], mn);
        if (nfw) atomicAdd(&c->nvisit_fw, nfw);
      }
      if (!step_sync(c, st, 28)) return;
      hit = w.bvis;
      hit_min = &c->minv[1];
    }
  }
  if (!together) {
    __syncthreads();
    if (!reach_multi<NC, kOptions>(&SF, 1, sflags, A, w, sm, st, ty)) return;
    const int32_t nf = (int32_t)SF.qhi;  // the whole forward set: no local rounds
    if (scc) {
      if (b == 0 && t == 0) atomicAdd(&c->nvisit_fw, nf);
      // backward inside the forward set; its candidates are the forward set
      B.allow = w.fvis;
      B.vis = w.bvis;
      B.cand = w.q;
      B.ncand = nf;
      B.minv = batch ? nullptr : &c->minv[1];
      if (t == 0) SB.R = B;
      __syncthreads();
      if (!reach_multi<1, kOptions>(&SB, 1, sflags, A, w, sm, st, ty)) return;
      hit = w.bvis;
      hit_min = &c->minv[1];
    } else {
      hit = w.fvis;
      hit_min = &c->minv[0];
    }
  }
  // batch: the smallest member of each graph's component labels it
  if (batch) {
    for (long long wd = (long long)b * T + t; wd < w.nwords; wd += (long long)G * T) {
      unsigned x = __ldcg(hit + wd);
      int32_t gprev = -1;
      while (x) {
        const int bit = __ffs(x) - 1;
        x &= x - 1;
        const int32_t v = (int32_t)(wd * 32 + bit);
        const int32_t gg = __ldg(g.batch.gid + v);
        if (gg != gprev) {  // bits rise, so v is the smallest of its graph here
          if (v < __ldcg(g.batch.gmin + gg)) atomicMin(g.batch.gmin + gg, v);
          gprev = gg;
        }
      }
    }
    if (!step_sync(c, st, 25)) return;
  }
  const int32_t lab = A.p.canonical ? (batch ? -1 : __ldcg(hit_min)) : pivot;
  // take the component out of the valid set (update_valid,
  // scc_fwbw.cpp:425-433) and label it while the valid list is compacted
  // (the component's size is counted here from its bitmap)
  int nhit = 0;
  for (long long wd = (long long)b * T + t; wd < w.nwords; wd += (long long)G * T) {
    const uint32_t h = __ldcg(hit + wd);
    if (h) {
      w.vbits[wd] = __ldcg(w.vbits + wd) & ~h;
      nhit += __popc(h);
    }
  }
  for (int o = 16; o; o >>= 1) nhit += __shfl_xor_sync(kFull, nhit, o);
  if (lane_id() == 0 && nhit) {
    atomicAdd(&c->nscc_fwbw, nhit);
    if (!scc) atomicAdd(&c->nvisit_fw, nhit);
  }
  const bool canon = A.p.canonical != 0;
  auto put = [&](int32_t v) {
    w.label[v] = batch ? (canon ? __ldcg(g.batch.gmin + __ldg(g.batch.gid + v)) : v) : lab;
  };
  trace_rec(c, nvalid, 12);
  if (!compact_ordered(w.listA, nvalid, w.listB, hit, w, sm, st, 26, &c->nvalid, ty, put)) return;
  if (!step_sync(c, st, 27)) return;
  const int32_t nv = __ldcg(&c->nvalid);
  for (long long i = (long long)b * T + t; i < nv; i += (long long)G * T) w.listA[i] = __ldcg(w.listB + i);
  trace_rec(c, nv, 15);
  tally_flush(ty, c, kKReach, A.p.count_unassigned != 0, sm.red_u);
  steps_close(c, st);
}

// ------------------------------------------------------------------------
// Colour phase: rounds of colour propagation until no vertex is left.
// SCC: each round propagates colours along out-edges to the fixed point;
// every vertex whose colour is its own id is a root; a backward search over
// same-colour vertices labels the root's SCC with the colour; the rest stay
// for the next round (scc_color, scc_color.cpp:340-373).  The reference
// hands the last <= vert_cutoff vertices to serial Tarjan; here the rounds
// simply continue to the end.  WCC: one propagation over the union
// adjacency; every vertex takes its colour as label (cc_color_propagate,
// cc_color.cpp:47-175).  Colours are minima (see ColourVisit), so a root is
// the smallest id of its SCC and every label is canonical.
// ------------------------------------------------------------------------
// Stops (before a round) after max_rounds rounds; *cur = the valid list
// then (listA or listB).
template <int NC>
__device__ void colour_rounds(const Args& A, Smem& sm, int max_rounds, int32_t** cur) {
  Work w = A.w;
  Ctl* c = w.ctl;
  const GraphView& g = A.g;
  const int G = gridDim.x, b = blockIdx.x, T = blockDim.x, t = threadIdx.x;
  const int warp = t >> 5;
  const long long gt = (long long)b * T + t, gstride = (long long)G * T;
  Tally ty;
  if (ld_vol(&c->err)) return;
  int32_t nl = __ldcg(&c->nvalid);
  if (nl == 0) return;
  Steps st = steps_open(c);
  const bool scc = A.kind == kSCC;
  const Adj prop = scc ? adj1(g.out) : adj_undirected(g);
  const Adj back = adj1(g.in);
  int32_t* L = w.listA;
  int32_t* L2 = w.listB;
  int rounds = 0;
  long long labelled = 0;
  int32_t* bufs[2] = {w.x0, w.x1};
  int32_t* hl[2] = {w.h0, w.h1};
  const Tune& tn = A.p.tune;
  *cur = L;
  while (nl > 0) {
    if (rounds >= max_rounds) break;
    if (rounds > g.n || st.s - st.s0 >= tn.max_steps) { set_err(c, kErrIterLimit, 30); return; }
    trace_rec(c, nl, 8);
    for (long long i = gt; i < nl; i += gstride) {
      const int32_t v = __ldcg(L + i);
      w.colour[v] = v;
      ty.list++;
    }
    if (!step_sync(c, st, 31)) return;
    // propagation; the first step pushes from every vertex of L
    {
      const int32_t* front = L;
      int32_t nfront = nl, nheavy = 0;
      int cur = 0, hs = 0;
      for (;;) {
        if (st.s - st.s0 >= tn.max_steps) { set_err(c, kErrIterLimit, 32); return; }
        trace_rec(c, nfront, 9);
        const ColourVisit cv{w.vbits, w.colour};
        const Sink sk = sink_make(bufs[cur], 0, w.n, step_out(c, st.s), false, nullptr,
                                  hl[hs ^ 1], w.n, 301);
        expand<NC>(front, nfront, hl[hs], nheavy, prop, cv, sk, tn, sm, c, ty);
        stat_inc(c, kStColourSteps);
        if (!step_sync(c, st, 33)) return;
        const StepIn in = step_read(c, st.s);
        if (in.count == 0 && in.huge == 0) break;
        front = bufs[cur];
        nfront = in.count;
        nheavy = in.huge;
        cur ^= 1;
        hs ^= 1;
      }
    }
    if (!scc) {
      for (long long i = gt; i < nl; i += gstride) {
        const int32_t v = __ldcg(L + i);
        w.label[v] = __ldcg(w.colour + v);
      }
      labelled += nl;
      nl = 0;
      ++rounds;
      break;
    }
    // roots: colour == own id (scc_color_get_roots, scc_color.cpp:179-201)
    const MarkVisit mv{w.vbits, w.done, w.colour, w.label};
    trace_rec(c, nl, 10);
    {
      Out ro;
      ro.arr = bufs[0];
      ro.base = 0;
      ro.cap = w.n;
      ro.counter = &step_out(c, st.s)->count;
      ro.edges = nullptr;
      ro.minv = nullptr;
      ro.where = 302;
      Stage rs = stage_make(sm.stage(warp, 0));
      for (long long base = gt - (t & 31); base < nl; base += gstride) {
        const long long i = base + (t & 31);
        bool root = false;
        int32_t v = 0;
        if (i < nl) {
          v = __ldcg(L + i);
          if (__ldcg(w.colour + v) == v && bit_claim(w.done, v)) {
            w.label[v] = v;
            root = true;
          }
        }
        stage_push(rs, root, v, 0ull, ro, c);
      }
      stage_flush(rs, ro, c);
      if (!step_sync(c, st, 34)) return;
    }
    // backward same-colour search from the roots
    {
      int cur = 0, hs = 0;
      for (;;) {
        if (st.s - st.s0 >= tn.max_steps) { set_err(c, kErrIterLimit, 35); return; }
        const StepIn in = step_read(c, st.s);
        if (in.count == 0 && in.huge == 0) break;
        trace_rec(c, in.count, 11);
        const Sink sk = sink_make(bufs[cur ^ 1], 0, w.n, step_out(c, st.s), false, nullptr,
                                  hl[hs ^ 1], w.n, 303);
        expand<1>(bufs[cur], in.count, hl[hs], in.huge, back, mv, sk, tn, sm, c, ty);
        stat_inc(c, kStMarkSteps);
        if (!step_sync(c, st, 36)) return;
        cur ^= 1;
        hs ^= 1;
      }
    }
    // the labelled vertices leave the valid set; L is compacted into L2
    trace_rec(c, nl, 12);
    auto release = [&](int32_t v) { bit_release(w.vbits, v); };
    if (!compact_ordered(L, nl, L2, w.done, w, sm, st, 37, &c->nvalid, ty, release)) return;
    if (!step_sync(c, st, 38)) return;
    const int32_t nn = __ldcg(&c->nvalid);
    labelled += nl - nn;
    nl = nn;
    int32_t* tmp = L;
    L = L2;
    L2 = tmp;
    *cur = L;
    ++rounds;
    stat_inc(c, kStColourRounds);
  }
  if (b == 0 && t == 0) {
    c->ncolour_rounds = rounds;
    c->ncolour = (int32_t)labelled;
  }
  trace_rec(c, 0, 15);
  tally_flush(ty, c, kKColour, A.p.count_unassigned != 0, sm.red_u);
  steps_close(c, st);
}

// ------------------------------------------------------------------------
// Signature rounds (colour_mode 1, or 2 on a large residual; SCC): each round,
// every valid vertex v gets fw[v], the smallest id that reaches it, and
// bw[v], the smallest id it reaches, both through edges inside its class
// (the vertices that carried the same (fw, bw) pair in the previous round;
// one class in the first round).  Members of one SCC share a class and a
// pair; a vertex whose two values agree reaches and is reached by that id,
// so it is in that vertex's SCC, whose smallest member it is: the label.
// The other vertices take their pair as their class (a 32-bit mix of it;
// a collision only merges classes), and no edge between classes is
// followed again.  Every class loses its smallest vertex's SCC each round,
// as a colour round does, but the classes split the residual into pieces
// whose propagations are short, and no backward marking search is needed.
// The labels are the colour rounds' (the minimum member of each SCC).
// ------------------------------------------------------------------------
__device__ __forceinline__ int32_t sig_class(int32_t f, int32_t b) {
  uint32_t x = (uint32_t)f * 0x9E3779B1u;
  x ^= (uint32_t)b * 0x85EBCA77u + 0x7F4A7C15u + (x << 6) + (x >> 2);
  return (int32_t)x;
}

// colour_mode 2: the signature rounds take a residual (valid vertices
// after FW-BW) of at least kSigMin vertices, and whatever kSigAfter colour
// rounds leave of a smaller one.
constexpr int32_t kSigMin = 1 << 20;
constexpr int kSigAfter = 4;

// (not inlined: its registers are allocated apart from the default run's
// hot loops)
__device__ __noinline__ void signature_rounds(const Args& A, Smem& sm, int32_t* L, int32_t* L2) {
  Work w = A.w;
  Ctl* c = w.ctl;
  const GraphView& g = A.g;
  const int G = gridDim.x, b = blockIdx.x, T = blockDim.x, t = threadIdx.x;
  const long long gt = (long long)b * T + t, gstride = (long long)G * T;
  Tally ty;
  if (ld_vol(&c->err)) return;
  int32_t nl = __ldcg(&c->nvalid);
  if (nl == 0) return;
  Steps st = steps_open(c);
  int32_t* fw = w.colour;
  int32_t* bw = w.live_in;
  int32_t* cls = w.live_out;
  const Adj outs = adj1(g.out), ins = adj1(g.in);
  int rounds = __ldcg(&c->ncolour_rounds);  // after colour rounds: continues their count
  int32_t labelled_before = __ldcg(&c->ncolour);
  long long labelled = 0;
  int32_t* bufs[2] = {w.x0, w.x1};
  int32_t* hl[2] = {w.h0, w.h1};
  const Tune& tn = A.p.tune;
  for (long long i = gt; i < nl; i += gstride) cls[__ldcg(L + i)] = 0;
  while (nl > 0) {
    if (rounds > g.n || st.s - st.s0 >= tn.max_steps) { set_err(c, kErrIterLimit, 40); return; }
    trace_rec(c, nl, 8);
    for (long long i = gt; i < nl; i += gstride) {
      const int32_t v = __ldcg(L + i);
      fw[v] = v;
      bw[v] = v;
      ty.list++;
    }
    if (!step_sync(c, st, 41)) return;
    // forward values along out-edges, then backward values along in-edges;
    // the first step of each pushes from every vertex of L
    for (int dir = 0; dir < 2; ++dir) {
      const SigVisit sv{w.vbits, dir == 0 ? fw : bw, cls};
      const Adj& a = dir == 0 ? outs : ins;
      const int32_t* front = L;
      int32_t nfront = nl, nheavy = 0;
      int cur = 0, hs = 0;
      for (;;) {
        if (st.s - st.s0 >= tn.max_steps) { set_err(c, kErrIterLimit, 42); return; }
        trace_rec(c, nfront, 9);
        const Sink sk = sink_make(bufs[cur], 0, w.n, step_out(c, st.s), false, nullptr,
                                  hl[hs ^ 1], w.n, 305);
        expand<1>(front, nfront, hl[hs], nheavy, a, sv, sk, tn, sm, c, ty);
        stat_inc(c, kStColourSteps);
        if (!step_sync(c, st, 43)) return;
        const StepIn in = step_read(c, st.s);
        if (in.count == 0 && in.huge == 0) break;
        front = bufs[cur];
        nfront = in.count;
        nheavy = in.huge;
        cur ^= 1;
        hs ^= 1;
      }
    }
    // a vertex whose two values agree is labelled; the others are reclassed
    trace_rec(c, nl, 10);
    for (long long i = gt; i < nl; i += gstride) {
      const int32_t v = __ldcg(L + i);
      const int32_t f = __ldcg(fw + v), bk = __ldcg(bw + v);
      if (f == bk) {
        w.label[v] = f;
        bit_claim(w.done, v);
      } else {
        cls[v] = sig_class(f, bk);
      }
    }
    if (!step_sync(c, st, 44)) return;
    trace_rec(c, nl, 12);
    auto release = [&](int32_t v) { bit_release(w.vbits, v); };
    if (!compact_ordered(L, nl, L2, w.done, w, sm, st, 45, &c->nvalid, ty, release)) return;
    if (!step_sync(c, st, 46)) return;
    const int32_t nn = __ldcg(&c->nvalid);
    labelled += nl - nn;
    nl = nn;
    int32_t* tmp = L;
    L = L2;
    L2 = tmp;
    ++rounds;
    stat_inc(c, kStColourRounds);
  }
  if (b == 0 && t == 0) {
    c->ncolour_rounds = rounds;
    c->ncolour = labelled_before + (int32_t)labelled;
  }
  trace_rec(c, 0, 15);
  tally_flush(ty, c, kKColour, A.p.count_unassigned != 0, sm.red_u);
  steps_close(c, st);
}

// Device time at a phase boundary (block 0, thread 0), into the run's slot
// of the context's phase-time ring.
__device__ __forceinline__ void phase_mark(const Args& A, int i) {
  if (blockIdx.x == 0 && threadIdx.x == 0 && A.w.tphase != nullptr) A.w.tphase[i] = gtimer();
}

// ------------------------------------------------------------------------
// k_run: one run (trim, reachability, colour rounds) in one cooperative
// launch; a grid barrier separates the phases, so each phase sees the
// previous one's lists, counters and pivot.  NC: adjacency lists walked by
// the reachability phase (1, or 2 for WCC of a directed graph).
// ------------------------------------------------------------------------
// kOptions: the optional features are compiled in: FW-BW rounds after the
// first, each from a new pivot while at least kRepivotMin vertices are valid
// (fwbw_rounds > 1, single graphs), and the edge-balanced push
// (expand_mode 1).  That variant is compiled in its own translation unit
// (kernels_options.cu), so the code of the default run is the same with or
// without it.
template <int NC, bool kOptions>
__global__ void __launch_bounds__(kBlock, kMinBlocks) k_run(Args A) {
  __shared__ Smem sm;
  sm.stage_base = g_dyn_smem;
  Ctl* c = A.w.ctl;
  phase_mark(A, 0);
  trim_phase(A, sm);
  if (!grid_barrier(c, 900)) return;
  phase_mark(A, 1);
  reach_phase<NC, false, kOptions>(A, sm);
  if constexpr (kOptions) {
    for (int r = 1; r < A.p.fwbw_rounds && A.g.batch.gid == nullptr; ++r) {
      if (!grid_barrier(c, 32)) return;  // the last round's valid count
      if (__ldcg(&c->nvalid) < kRepivotMin) break;
      if (!repivot(A, sm)) return;
      if (__ldcg(&c->rpivot) < 0) break;
      reach_phase<NC, true, true>(A, sm);
    }
  }
  if (!grid_barrier(c, 901)) return;
  phase_mark(A, 2);
  // (every block reads the same counts after a barrier, so all take the
  // same branches)
  const bool scc = A.kind == kSCC;
  if (scc && (A.p.colour_mode == 1 || (A.p.colour_mode == 2 && __ldcg(&c->nvalid) >= kSigMin))) {
    signature_rounds(A, sm, A.w.listA, A.w.listB);
  } else {
    // colour_mode 2: a residual still left after kSigAfter colour rounds
    // goes on in signature rounds (a deep condensation: chains)
    const int cap = scc && A.p.colour_mode == 2 ? kSigAfter : 0x7fffffff;
    int32_t* cur = A.w.listA;
    if (scc || A.g.in.off == nullptr) colour_rounds<1>(A, sm, cap, &cur);
    else colour_rounds<2>(A, sm, cap, &cur);
    if (cap != 0x7fffffff) {
      if (!grid_barrier(c, 903)) return;
      if (__ldcg(&c->nvalid) > 0 && !ld_vol(&c->err))
        signature_rounds(A, sm, cur, cur == A.w.listA ? A.w.listB : A.w.listA);
    }
  }
  if (!grid_barrier(c, 902)) return;
  phase_mark(A, 3);
}

template <class K>
cudaError_t coop(K kern, int grid, const Args& a, cudaStream_t s) {
  void* params[] = {const_cast<Args*>(&a)};
  return cudaLaunchCooperativeKernel((const void*)kern, dim3(grid), dim3(kBlock), params,
                                     (size_t)kDynSmem, s);
}

// Blocks per SM of a run kernel at kDynSmem bytes of dynamic shared memory
// (0 on an error).
template <class K>
int run_blocks_per_sm(K kern) {
  if (cudaFuncSetAttribute((const void*)kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           kDynSmem) != cudaSuccess)
    return 0;
  int per = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, (const void*)kern, kBlock, kDynSmem) !=
      cudaSuccess)
    return 0;
  return per;
}

}  // namespace
}  // namespace gb
