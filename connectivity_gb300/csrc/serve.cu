// Serving: a request loop over one GPU with continuous batching.
//
// Clients submit graphs (edge lists in host memory) with an arrival time;
// the engine thread admits every arrived request that fits the device-memory
// budget, merges the admitted graphs into one SCC union and one WCC union
// (the batch path, batch.cu), runs them, and hands each request its labels.
// While one set of merged graphs runs on the compute stream, the edges of
// the requests admitted next are already being copied to the device on a
// copy stream, so new arrivals are taken in between runs and their transfer
// overlaps the running work.  Graph state (CSR, hints, labels) lives in the
// stream-ordered device pool for as long as its request is in flight.  Each
// request's labels are the ones it gets alone (the batch path guarantees
// it); latency is completion minus arrival on the server clock.
//
// A merged set of up to kSmallWave requests that are all small (at most
// kSmallMaxN vertices and kSmallAutoEdges edges each) skips the union
// build: each request runs in one thread block straight from its uploaded
// edges (small.cu), all of them in one launch, so at low and moderate load a
// request costs one short launch instead of a radix-sort CSR build and a
// cooperative run.  Any other set takes the union path as a whole.
//
// The reference has no serving; its equivalent is one run_scc / run_cc call
// per request (multistep/scc_main.cpp:210, cc_main.cpp:184).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/gbconn.h"
#include "api_internal.h"
#include "gb_internal.cuh"
#include "host_internal.h"

namespace {

// Adds each graph's vertex base to its edges' ids (edges of graph g are
// [eb[g], eb[g+1]), its vertices [vb[g], vb[g+1])).  An id outside the
// graph marks the graph bad and its edge becomes a self-loop on the graph's
// first vertex, so the other graphs of the merged run are unaffected.
__global__ void k_offset_ids(int32_t* src, int32_t* dst, int64_t m, const int64_t* eb,
                             const int64_t* vb, int32_t count, int32_t* bad) {
  constexpr int kRunLen = 64;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r * kRunLen < m;
       r += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = r * kRunLen;
    const int64_t end = i + kRunLen < m ? i + kRunLen : m;
    int lo = 0, hi = count;
    while (hi - lo > 1) {
      const int mid = (lo + hi) / 2;
      if (eb[mid] <= i) lo = mid; else hi = mid;
    }
    int g = lo;
    for (; i < end; ++i) {
      while (g + 1 < count && eb[g + 1] <= i) ++g;
      const int32_t base = (int32_t)vb[g];
      const int32_t ng = (int32_t)(vb[g + 1] - vb[g]);
      int32_t a = src[i], b = dst[i];
      if (a < 0 || a >= ng || b < 0 || b >= ng) {
        bad[g] = 1;
        a = b = 0;
      }
      src[i] = a + base;
      dst[i] = b + base;
    }
  }
}

struct Req {
  int64_t id = 0;
  int kind = 0;  // 0 SCC, 1 WCC
  int32_t n = 0;
  int64_t m = 0;
  const int32_t* src = nullptr;
  const int32_t* dst = nullptr;
  int32_t* out = nullptr;
  int64_t arrival_ns = 0;
  int64_t done_ns = -1;
  int64_t bytes = 0;
  int status = GB_OK;
  bool done = false;
};

// One merged set of graphs of one kind.
struct Part {
  std::vector<Req*> reqs;
  std::vector<int64_t> vbase, ebase;
  int64_t n = 0, m = 0;
  int32_t* d_src = nullptr;
  int32_t* d_dst = nullptr;
  int64_t* d_eb = nullptr;
  int64_t* d_vb = nullptr;
  int32_t* h_labels = nullptr;  // pinned
  size_t h_cap = 0;
  int32_t* d_bad = nullptr;     // per-graph id check
  int32_t* h_bad = nullptr;     // pinned
  size_t h_bad_cap = 0;
  int32_t* d_labels = nullptr;
  gb_batch* batch = nullptr;
  int32_t nlarge = 0;             // requests on the union path (listed first)
  gb::SmallDesc* d_descs = nullptr;  // the one-block requests
  int32_t* d_scratch = nullptr;      // their CSRs (SCC)
};

// A set of small requests runs one block each when it has at most this
// many (two waves of one block per SM); a larger set goes to the union.
constexpr int32_t kSmallWave = 304;

struct Flight {
  Part part[2];
  cudaEvent_t uploaded = nullptr;
  cudaEvent_t done = nullptr;
  bool active = false;
  int64_t bytes = 0;
  int status = GB_OK;
};

int64_t request_bytes(int32_t n, int64_t m) {
  // CSR (two offset arrays, two adjacency arrays), hints, staged edges,
  // labels and the per-vertex workspace share
  return (int64_t)n * (16 + 8 + 4 + 64) + m * (8 + 8) + 4096;
}

}  // namespace

struct gb_server {
  gb_ctx* ctx = nullptr;
  gb_opts opts{};   // options of the merged runs
  bool opts_set = false;  // set by gb_server_set_opts; otherwise the context's
                          // class table (if any) picks per merged set
  cudaStream_t copy = nullptr;
  int64_t budget = 0;
  int32_t max_graphs = 0;
  std::thread th;
  std::mutex mu;
  std::condition_variable cv;       // engine wake-up
  std::condition_variable done_cv;  // request completion
  std::deque<Req*> pending;         // arrival order
  std::unordered_map<int64_t, Req*> reqs;
  int64_t next_id = 1;
  bool stop = false;
  bool started = false;
  std::chrono::steady_clock::time_point t0;
  int64_t inflight_bytes = 0;
  Flight fl[2];
  int cur = 0;
  // statistics
  int64_t completed = 0, batches = 0, merged_graphs = 0;
  int64_t first_arrival = -1, last_done = -1;
  std::vector<int64_t> latencies;
  int last_error = GB_OK;

  int64_t now_ns() const {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now() - t0)
        .count();
  }
};

namespace {

void part_release(gb_server* sv, Part& p) {
  cudaStream_t s = sv->ctx->stream;
  if (p.batch) gb_batch_destroy(p.batch);
  p.batch = nullptr;
  if (p.d_src) cudaFreeAsync(p.d_src, s);
  if (p.d_dst) cudaFreeAsync(p.d_dst, s);
  if (p.d_eb) cudaFreeAsync(p.d_eb, s);
  if (p.d_vb) cudaFreeAsync(p.d_vb, s);
  if (p.d_labels) cudaFreeAsync(p.d_labels, s);
  if (p.d_bad) cudaFreeAsync(p.d_bad, s);
  if (p.d_descs) cudaFreeAsync(p.d_descs, s);
  if (p.d_scratch) cudaFreeAsync(p.d_scratch, s);
  p.d_descs = nullptr;
  p.d_scratch = nullptr;
  p.nlarge = 0;
  p.d_bad = nullptr;
  p.d_src = p.d_dst = nullptr;
  p.d_eb = p.d_vb = nullptr;
  p.d_labels = nullptr;
  p.reqs.clear();
  p.n = p.m = 0;
}

// Copies the admitted requests' edges to the device (copy stream).  The
// requests that take the union path come first.
gb_status part_upload(gb_server* sv, Part& p) {
  // all small and few: one block each; otherwise one union run for all
  // (a union run and a one-block launch of the same set would run one
  // after the other, and the set's latency would be their sum)
  bool all_small = sv->opts.small_path && sv->opts.canonical &&
                   (int32_t)p.reqs.size() <= kSmallWave;
  for (const Req* r : p.reqs)
    if (!(r->n <= gb::kSmallMaxN && r->m <= gb::kSmallAutoEdges)) all_small = false;
  p.nlarge = all_small ? 0 : (int32_t)p.reqs.size();
  p.vbase.assign(1, 0);
  p.ebase.assign(1, 0);
  for (Req* r : p.reqs) {
    p.vbase.push_back(p.vbase.back() + r->n);
    p.ebase.push_back(p.ebase.back() + r->m);
  }
  p.n = p.vbase.back();
  p.m = p.ebase.back();
  const size_t eb = (size_t)(p.m > 0 ? p.m : 1) * 4;
  cudaStream_t cs = sv->copy;
  if (cudaMallocAsync(&p.d_src, eb, cs) != cudaSuccess || cudaMallocAsync(&p.d_dst, eb, cs) != cudaSuccess ||
      cudaMallocAsync(&p.d_eb, p.ebase.size() * 8, cs) != cudaSuccess ||
      cudaMallocAsync(&p.d_vb, p.vbase.size() * 8, cs) != cudaSuccess ||
      cudaMallocAsync(&p.d_bad, p.reqs.size() * 4, cs) != cudaSuccess)
    return GB_ERR_OOM;
  if (cudaMemsetAsync(p.d_bad, 0, p.reqs.size() * 4, cs) != cudaSuccess) return GB_ERR_CUDA;
  for (size_t i = 0; i < p.reqs.size(); ++i) {
    const Req* r = p.reqs[i];
    if (r->m == 0) continue;
    if (cudaMemcpyAsync(p.d_src + p.ebase[i], r->src, (size_t)r->m * 4, cudaMemcpyHostToDevice, cs) !=
            cudaSuccess ||
        cudaMemcpyAsync(p.d_dst + p.ebase[i], r->dst, (size_t)r->m * 4, cudaMemcpyHostToDevice, cs) !=
            cudaSuccess)
      return GB_ERR_CUDA;
  }
  if (cudaMemcpyAsync(p.d_eb, p.ebase.data(), p.ebase.size() * 8, cudaMemcpyHostToDevice, cs) !=
          cudaSuccess ||
      cudaMemcpyAsync(p.d_vb, p.vbase.data(), p.vbase.size() * 8, cudaMemcpyHostToDevice, cs) !=
          cudaSuccess)
    return GB_ERR_CUDA;
  // (the pinned buffers are sized at creation and grow by half again when
  // a merged set outgrows them: pinning inside the request stream stalls it)
  if ((size_t)p.n > p.h_cap) {
    if (p.h_labels) cudaFreeHost(p.h_labels);
    p.h_labels = nullptr;
    const size_t want = std::max((size_t)p.n, p.h_cap * 3 / 2);
    p.h_cap = 0;
    if (cudaMallocHost(&p.h_labels, want * 4) != cudaSuccess) return GB_ERR_OOM;
    p.h_cap = want;
  }
  if (p.reqs.size() > p.h_bad_cap) {
    if (p.h_bad) cudaFreeHost(p.h_bad);
    p.h_bad = nullptr;
    p.h_bad_cap = 0;
    if (cudaMallocHost(&p.h_bad, p.reqs.size() * 4) != cudaSuccess) return GB_ERR_OOM;
    p.h_bad_cap = p.reqs.size();
  }
  return GB_OK;
}

// Pinned host buffers of every part, sized before the server starts.
constexpr size_t kInitLabels = size_t(1) << 22;  // labels per part (16 MB)
gb_status reserve_parts(gb_server* sv) {
  for (auto& f : sv->fl)
    for (auto& p : f.part) {
      if (cudaMallocHost(&p.h_labels, kInitLabels * 4) != cudaSuccess) return GB_ERR_OOM;
      p.h_cap = kInitLabels;
      if (cudaMallocHost(&p.h_bad, (size_t)sv->max_graphs * 4) != cudaSuccess) return GB_ERR_OOM;
      p.h_bad_cap = (size_t)sv->max_graphs;
    }
  return GB_OK;
}

// Builds the merged graph and queues its run (compute stream; the build
// itself waits for the stream).
gb_status part_launch(gb_server* sv, Part& p, int kind) {
  gb_ctx* c = sv->ctx;
  cudaStream_t s = c->stream;
  const int32_t count = (int32_t)p.reqs.size();
  if (count == 0) return GB_OK;
  if (p.m > 0) {
    long long blocks = (p.m / 64 + 255) / 256 + 1;
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_offset_ids<<<(int)blocks, 256, 0, s>>>(p.d_src, p.d_dst, p.m, p.d_eb, p.d_vb, count, p.d_bad);
    if (cudaGetLastError() != cudaSuccess) return GB_ERR_CUDA;
  }
  if (cudaMemcpyAsync(p.h_bad, p.d_bad, (size_t)count * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return GB_ERR_CUDA;
  // grow the context workspace (the union run's) ahead of need, so it is
  // rarely reallocated
  const int64_t n_union = p.vbase[(size_t)p.nlarge];
  if (p.nlarge > 0 && n_union > c->cap_n) {
    int64_t want = std::max<int64_t>(n_union, (int64_t)c->cap_n * 3 / 2);
    if (want > 0x7fffffffll) want = 0x7fffffffll;
    gb_status ws = gb::reserve_workspace(c, (int32_t)want);
    if (ws != GB_OK) return ws;
  }
  if (cudaMallocAsync(&p.d_labels, (size_t)(p.n > 0 ? p.n : 1) * 4, s) != cudaSuccess) return GB_ERR_OOM;
  if (p.nlarge > 0) {
    gb_status st = gb::batch_create(c, p.nlarge, p.vbase.data(), p.ebase[(size_t)p.nlarge],
                                    p.d_src, p.d_dst, false, true, &p.batch);
    if (st != GB_OK) return st;
    const gb_opts* po = sv->opts_set ? nullptr : gb::class_opts(c, p.vbase[(size_t)p.nlarge]);
    st = gb::batch_run(c, p.batch, kind == 0 ? gb::kSCC : gb::kWCC, p.d_labels,
                       po ? po : &sv->opts, nullptr, false);
    if (st != GB_OK) return st;
  }
  if (p.nlarge < count) {
    // one block per small request, from its edges (global ids: id_base)
    const int32_t ns = count - p.nlarge;
    const int64_t e0 = p.ebase[(size_t)p.nlarge];
    const int64_t ms = p.m - e0;
    if (kind == 0 && ms > 0 &&
        cudaMallocAsync(&p.d_scratch, (size_t)ms * 8, s) != cudaSuccess)
      return GB_ERR_OOM;
    std::vector<gb::SmallDesc> h((size_t)ns);
    int32_t max_n = 1;
    for (int32_t i = 0; i < ns; ++i) {
      const size_t g = (size_t)(p.nlarge + i);
      gb::SmallDesc& d = h[(size_t)i];
      d.n = (int32_t)(p.vbase[g + 1] - p.vbase[g]);
      d.id_base = (int32_t)p.vbase[g];
      d.m = p.ebase[g + 1] - p.ebase[g];
      d.src = p.d_src + p.ebase[g];
      d.dst = p.d_dst + p.ebase[g];
      d.adj_scratch = kind == 0 ? p.d_scratch + 2 * (p.ebase[g] - e0) : nullptr;
      d.labels = p.d_labels + p.vbase[g];
      max_n = std::max(max_n, d.n);
    }
    if (cudaMallocAsync(&p.d_descs, (size_t)ns * sizeof(gb::SmallDesc), s) != cudaSuccess)
      return GB_ERR_OOM;
    // (pageable source: the copy is staged before the call returns)
    if (cudaMemcpyAsync(p.d_descs, h.data(), (size_t)ns * sizeof(gb::SmallDesc),
                        cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(&c->d_ctl->err, 0, 2 * sizeof(int), s) != cudaSuccess)
      return GB_ERR_CUDA;
    const int32_t max_steps = sv->opts.max_steps > 0 ? sv->opts.max_steps : (1 << 30);
    if (gb::launch_small(kind, h[0], p.d_descs, ns, max_n, max_steps, &c->d_ctl->err, s,
                         sv->opts.colour_mode) !=
            cudaSuccess ||
        gb::launch_latch(c->d_ctl, c->d_sticky, s) != cudaSuccess)
      return GB_ERR_CUDA;
  }
  if (p.n > 0 &&
      cudaMemcpyAsync(p.h_labels, p.d_labels, (size_t)p.n * 4, cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return GB_ERR_CUDA;
  return GB_OK;
}

void finish_flight(gb_server* sv, Flight& f) {
  gb_status st = f.status;
  cudaError_t e = cudaEventSynchronize(f.done);
  if (st == GB_OK && e != cudaSuccess) st = gb::cuda_fail(e, "serve");
  if (st == GB_OK) st = gb_ctx_sync(sv->ctx);
  const int64_t t = sv->now_ns();
  std::unique_lock<std::mutex> lk(sv->mu);
  for (int k = 0; k < 2; ++k) {
    Part& p = f.part[k];
    for (size_t i = 0; i < p.reqs.size(); ++i) {
      Req* r = p.reqs[i];
      gb_status rs = st;
      if (rs == GB_OK && p.h_bad[i]) rs = GB_ERR_INVALID;
      if (rs == GB_OK && r->out && r->n > 0)
        std::memcpy(r->out, p.h_labels + p.vbase[i], (size_t)r->n * 4);
      r->status = rs;
      r->done_ns = t;
      r->done = true;
      sv->completed++;
      sv->latencies.push_back(t - r->arrival_ns);
      if (sv->first_arrival < 0 || r->arrival_ns < sv->first_arrival) sv->first_arrival = r->arrival_ns;
      sv->last_done = t;
    }
  }
  if (st != GB_OK) sv->last_error = st;
  sv->inflight_bytes -= f.bytes;
  lk.unlock();
  for (int k = 0; k < 2; ++k) part_release(sv, f.part[k]);
  f.active = false;
  f.bytes = 0;
  f.status = GB_OK;
  sv->done_cv.notify_all();
}

void engine(gb_server* sv) {
  cudaSetDevice(sv->ctx->device);
  for (;;) {
    Flight& nxt = sv->fl[sv->cur ^ 1];
    Flight& run = sv->fl[sv->cur];
    // admit the requests that have arrived and fit
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      const int64_t now = sv->now_ns();
      int32_t taken = 0;
      int64_t bytes = 0;
      while (!sv->pending.empty() && taken < sv->max_graphs) {
        Req* r = sv->pending.front();
        if (r->arrival_ns > now) break;
        if (sv->inflight_bytes + bytes + r->bytes > sv->budget && (taken > 0 || run.active)) break;
        sv->pending.pop_front();
        nxt.part[r->kind].reqs.push_back(r);
        bytes += r->bytes;
        ++taken;
      }
      sv->inflight_bytes += bytes;
      nxt.bytes = bytes;
      if (taken == 0 && !run.active) {
        if (sv->stop && sv->pending.empty()) return;
        // sleep until the next arrival, a submit or a stop
        if (sv->pending.empty()) {
          sv->cv.wait_for(lk, std::chrono::milliseconds(50));
        } else {
          const int64_t wait = sv->pending.front()->arrival_ns - sv->now_ns();
          if (wait > 20000) sv->cv.wait_for(lk, std::chrono::nanoseconds(wait - 10000));
        }
        continue;
      }
      if (taken > 0) {
        sv->batches++;
        sv->merged_graphs += taken;
      }
    }
    const bool have_next = !nxt.part[0].reqs.empty() || !nxt.part[1].reqs.empty();
    // start the next transfers while the running set computes
    if (have_next) {
      for (int k = 0; k < 2 && nxt.status == GB_OK; ++k)
        if (!nxt.part[k].reqs.empty()) nxt.status = part_upload(sv, nxt.part[k]);
      cudaEventRecord(nxt.uploaded, sv->copy);
    }
    if (run.active) finish_flight(sv, run);
    if (have_next) {
      if (nxt.status == GB_OK) {
        cudaStreamWaitEvent(sv->ctx->stream, nxt.uploaded, 0);
        for (int k = 0; k < 2 && nxt.status == GB_OK; ++k)
          nxt.status = part_launch(sv, nxt.part[k], k);
      }
      cudaEventRecord(nxt.done, sv->ctx->stream);
      nxt.active = true;
      sv->cur ^= 1;
    }
  }
}

}  // namespace

extern "C" {

gb_status gb_server_create(gb_ctx* ctx, int64_t budget_bytes, int32_t max_graphs,
                           gb_server** out) {
  if (!ctx || !out || max_graphs < 1) return GB_ERR_INVALID;
  *out = nullptr;
  if (cudaSetDevice(ctx->device) != cudaSuccess) return GB_ERR_CUDA;
  if (budget_bytes <= 0) {
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return GB_ERR_CUDA;
    budget_bytes = (int64_t)(fr / 2);
  }
  gb_server* sv = new (std::nothrow) gb_server();
  if (!sv) return GB_ERR_OOM;
  sv->ctx = ctx;
  gb_opts_default(&sv->opts);
  sv->budget = budget_bytes;
  sv->max_graphs = max_graphs;
  // freed graph memory stays in the pool for the next requests
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) {
    uint64_t thr = (uint64_t)budget_bytes;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  if (cudaStreamCreateWithFlags(&sv->copy, cudaStreamNonBlocking) != cudaSuccess) {
    delete sv;
    return GB_ERR_CUDA;
  }
  for (auto& f : sv->fl) {
    cudaEventCreateWithFlags(&f.uploaded, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&f.done, cudaEventDisableTiming);
  }
  if (reserve_parts(sv) != GB_OK) {
    gb_server_destroy(sv);
    return GB_ERR_OOM;
  }
  *out = sv;
  return GB_OK;
}

gb_status gb_server_set_opts(gb_server* sv, const gb_opts* o) {
  if (!sv || !o) return GB_ERR_INVALID;
  std::lock_guard<std::mutex> lk(sv->mu);
  if (sv->started) return GB_ERR_INVALID;
  sv->opts = *o;
  sv->opts_set = true;
  return GB_OK;
}

gb_status gb_server_start(gb_server* sv) {
  if (!sv) return GB_ERR_INVALID;
  std::lock_guard<std::mutex> lk(sv->mu);
  if (sv->started) return GB_OK;
  sv->t0 = std::chrono::steady_clock::now();
  sv->started = true;
  sv->th = std::thread(engine, sv);
  return GB_OK;
}

gb_status gb_server_submit(gb_server* sv, int32_t kind, int32_t n, int64_t m, const int32_t* src,
                           const int32_t* dst, int32_t* labels_out, int64_t arrival_ns,
                           int64_t* id) {
  // edge ids are checked on the device (k_offset_ids): a request with an id
  // outside [0, n) completes with GB_ERR_INVALID
  if (!sv || (kind != 0 && kind != 1) || n < 1 || m < 0 || (m > 0 && (!src || !dst)) || !labels_out)
    return GB_ERR_INVALID;
  Req* r = new (std::nothrow) Req();
  if (!r) return GB_ERR_OOM;
  r->kind = kind;
  r->n = n;
  r->m = m;
  r->src = src;
  r->dst = dst;
  r->out = labels_out;
  r->bytes = request_bytes(n, m);
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    if (r->bytes > sv->budget) {
      delete r;
      gb_set_error("gb_server_submit: %s", "request larger than the device-memory budget");
      return GB_ERR_CAPACITY;
    }
    r->id = sv->next_id++;
    r->arrival_ns = arrival_ns >= 0 ? arrival_ns : (sv->started ? sv->now_ns() : 0);
    // keep the queue in arrival order
    auto it = sv->pending.end();
    while (it != sv->pending.begin() && (*(it - 1))->arrival_ns > r->arrival_ns) --it;
    sv->pending.insert(it, r);
    sv->reqs[r->id] = r;
    if (id) *id = r->id;
  }
  sv->cv.notify_all();
  return GB_OK;
}

gb_status gb_server_wait(gb_server* sv, int64_t id, int64_t* latency_ns) {
  if (!sv) return GB_ERR_INVALID;
  std::unique_lock<std::mutex> lk(sv->mu);
  auto it = sv->reqs.find(id);
  if (it == sv->reqs.end()) return GB_ERR_INVALID;
  Req* r = it->second;
  sv->done_cv.wait(lk, [&] { return r->done; });
  if (latency_ns) *latency_ns = r->done_ns - r->arrival_ns;
  return r->status;
}

gb_status gb_server_drain(gb_server* sv) {
  if (!sv) return GB_ERR_INVALID;
  std::unique_lock<std::mutex> lk(sv->mu);
  sv->done_cv.wait(lk, [&] { return sv->completed == sv->next_id - 1; });
  return sv->last_error;
}

gb_status gb_server_stats_get(gb_server* sv, gb_server_stats* out) {
  if (!sv || !out) return GB_ERR_INVALID;
  std::lock_guard<std::mutex> lk(sv->mu);
  std::memset(out, 0, sizeof(*out));
  out->completed = sv->completed;
  out->batches = sv->batches;
  out->mean_batch = sv->batches ? (double)sv->merged_graphs / (double)sv->batches : 0.0;
  std::vector<int64_t> l = sv->latencies;
  std::sort(l.begin(), l.end());
  if (!l.empty()) {
    out->p50_ms = l[(l.size() - 1) / 2] / 1e6;
    out->p99_ms = l[(size_t)((l.size() - 1) * 0.99)] / 1e6;
    out->max_ms = l.back() / 1e6;
  }
  const int64_t span = sv->last_done - sv->first_arrival;
  out->graphs_per_s = span > 0 ? (double)sv->completed / (span / 1e9) : 0.0;
  return GB_OK;
}

gb_status gb_server_destroy(gb_server* sv) {
  if (!sv) return GB_OK;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
  }
  sv->cv.notify_all();
  if (sv->th.joinable()) sv->th.join();
  cudaSetDevice(sv->ctx->device);
  for (auto& f : sv->fl) {
    if (f.active) finish_flight(sv, f);
    for (auto& p : f.part) {
      part_release(sv, p);
      if (p.h_labels) cudaFreeHost(p.h_labels);
      if (p.h_bad) cudaFreeHost(p.h_bad);
    }
    cudaEventDestroy(f.uploaded);
    cudaEventDestroy(f.done);
  }
  cudaStreamSynchronize(sv->ctx->stream);
  cudaStreamDestroy(sv->copy);
  for (auto& kv : sv->reqs) delete kv.second;
  delete sv;
  return GB_OK;
}

}  // extern "C"
